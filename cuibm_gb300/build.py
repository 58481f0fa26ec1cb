"""Build libcuibm_gb300.so in-tree (cuibm_gb300/_lib/) with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into one shared
library that exports the C ABI declared in include/cuibm.h.  Host code is built
with -ffp-contract=off: grid and body coordinates must be bit-identical to the
reference's (no fused multiply-add on either x86-64 or aarch64 hosts).  The
immersed-boundary kernels are built with -fmad=false so that their tag
decisions follow the reference's arithmetic exactly.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB = os.path.join(LIB_DIR, "libcuibm_gb300.so")
CLI = os.path.join(LIB_DIR, "cuibm")  # the command-line program (csrc/cli.cpp) on the C ABI

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-Wall,-Wno-unused-function",
          "-I" + os.path.join(HERE, "..", "include")]
# translation unit -> extra flags
UNITS = {
    "config.cpp": [],
    "geometry.cpp": [],
    "fields.cpp": [],
    "io.cpp": [],
    "batch.cpp": [],
    "context.cu": [],
    "ns_kernels.cu": [],
    "krylov.cu": [],
    "amg.cu": [],
    "fused_solve.cu": [],
    "fused_op1.cu": [],
    "fused_op2.cu": [],
    "fused_mixed_op1.cu": [],
    "fused_mixed_op2.cu": [],
    "adjoint.cu": [],
    "fadlun.cu": ["-fmad=false"],
    "embedded.cu": ["-fmad=false"],
    "ib_kernels.cu": ["-fmad=false"],
}


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _compile(unit, flags):
    src = os.path.join(SRC, unit)
    obj = os.path.join(OBJ_DIR, unit + ".o")
    deps = [src] + [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "cuibm.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", src, "-o", obj]
    if unit.endswith(".cpp"):
        cmd = [nvcc()] + COMMON + flags + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stdout + r.stderr))
    return obj


def build(verbose=False):
    os.makedirs(OBJ_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), UNITS.items()))
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs)):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stdout + r.stderr))
    cli_src = os.path.join(SRC, "cli.cpp")
    if not (os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(LIB), os.path.getmtime(cli_src))):
        cmd = [nvcc()] + COMMON + [cli_src, "-o", CLI, "-L" + LIB_DIR, "-lcuibm_gb300", "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("cli build failed:\n%s\n%s" % (" ".join(cmd), r.stdout + r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    try:
        build(verbose=True)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
