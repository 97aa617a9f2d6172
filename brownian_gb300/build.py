"""Build recipe for the sm_103a libraries (in-tree, no cmake).

    python -m brownian_gb300.build          # or brownian_gb300.build.build()

Compiles the CUDA translation units in parallel with nvcc for sm_103a and links
lib/libbrownian_gb300.so (the C ABI of include/brownian_gb300.h) and
lib/libbrownian_shim.so (the reference's routine symbols over the C ABI).
Host code is compiled with -ffp-contract=off so host-side FP64 (initial
placement, derived constants) rounds like the reference's x86-64 build on any
host architecture.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libbrownian_gb300.so")
SHIM = os.path.join(OUT, "libbrownian_shim.so")

SOURCES = ["kernels_fp64.cu", "kernels_fp32c.cu", "init_fp64.cu", "context.cu", "noalloc.cu", "mlp.cu", "surrogate.cu",
           "diag.cu", "traj.cu", "routines.cu"]
SHIM_SOURCES = ["shim.cpp"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--extended-lambda", "-lineinfo",
              "-Xcompiler", "-fPIC,-ffp-contract=off"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the sm_103a build needs the CUDA toolkit")


def _deps():
    hdr = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".inc", ".h"))]
    hdr.append(os.path.join(ROOT, "include", "brownian_gb300.h"))
    return max(os.path.getmtime(h) for h in hdr)


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources) or _deps() > t


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(verbose=False, force=False):
    """Compile what changed; returns the path of libbrownian_gb300.so."""
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src]):
            jobs.append([cc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                print(r.stdout + r.stderr, end="")
    if force or jobs or not os.path.exists(LIB):
        _run([cc, "-shared", "-o", LIB] + objs)
    shim_src = [os.path.join(CSRC, s) for s in SHIM_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if shim_src and (force or _stale(SHIM, shim_src + [LIB])):
        _run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-o", SHIM]
             + shim_src + ["-L" + OUT, "-lbrownian_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)
