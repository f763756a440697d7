"""In-tree build of libhydro_gpu.so (nvcc, sm_103a only) and of the CPU
oracle (test infrastructure, oracle/Makefile).

    python -m hydro_gb300.build          # both
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["fluid.cu", "linear.cu", "mg.cu", "advection.cu", "control.cu", "context.cu", "heat.cu",
           "conv.cu", "net.cu", "desc.cpp",
           "noalloc.cu", "output.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")  # .cu and host-only .cpp
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    inc = os.path.join(ROOT, "include")
    deps += [os.path.join(inc, h) for h in os.listdir(inc) if h.endswith(".h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def build_library(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    out = os.path.join(HERE, "libhydro_gpu.so")
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", out] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", out)
    return out


def build_oracle():
    """CPU oracle (and the reference harness where the reference tree is
    present) -- test infrastructure, never linked into the library."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


def build(verbose=False):
    lib = build_library(verbose)
    build_oracle()
    return lib


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
