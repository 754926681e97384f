"""Build the CUDA library libsalsa_gb300.so in-tree for sm_103a.

The kernel forms (FP64 / FP32-mixed x with / without diagnostics, and the two
secondary-ice forms) are separate translation units so they compile in parallel.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsalsa_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
UNITS = ["salsa_k_d0.cu", "salsa_k_d1.cu", "salsa_k_f0.cu", "salsa_k_f1.cu", "salsa_k_ds.cu", "salsa_k_fs.cu",
         "salsa_chain.cu", "salsa_post.cu", "salsa_sedim.cu", "salsa_capi.cu"]
# Units compiled without multiply-add contraction, so that their arithmetic rounds
# like the reference's x86-64 SSE2 build: the post-step constraints, which match the
# oracle bit for bit.  The step kernels (both forms), the gradient harness (whose
# forward step is the step kernel's) and the sedimentation contract multiply-adds; the
# step's ice-nucleation arithmetic keeps its products unfused with explicit
# round-to-nearest multiplies.
FP64_UNITS = ("salsa_post.cu",)


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))] + \
        [os.path.join(HERE, "..", "include", "salsa_gb300.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources()) and os.path.getmtime(__file__) <= t


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(u):
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        extra = ["-fmad=false"] if u in FP64_UNITS else []
        cmd = [cc] + ARCH + FLAGS + extra + ["-c", os.path.join(CSRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stdout}\n{r.stderr}")
        with open(os.path.join(BUILD, u + ".ptxas.txt"), "w") as fh:
            fh.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
