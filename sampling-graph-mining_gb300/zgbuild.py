"""Build step for libzgraph_gpu.so (sm_103a) and the CPU oracle library.

Compiles every translation unit of csrc/ with nvcc in parallel (one -gencode, sm_103a only)
and links one shared library in-tree at sampling-graph-mining_gb300/_build/.  The oracle
(test infrastructure) is compiled with gcc into oracle/_build/.  No cmake; a minute or two
on a cold machine.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libzgraph_gpu.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "libzgoracle.so")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
                        "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_library(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "zgraph_gpu.h"))
    units = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    objs, jobs = [], []
    for u in units:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or _stale(LIB, objs):
        _run([nvcc] + GENCODE + ["-shared", "-o", LIB] + objs)
    return LIB


def build_oracle(verbose=False, force=False):
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    src = os.path.join(ORACLE_DIR, "zg_oracle.c")
    deps = [src, os.path.join(ORACLE_DIR, "zg_oracle.h"), os.path.join(ROOT, "include", "zgraph_gpu.h")]
    if force or _stale(ORACLE_LIB, deps):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O2", "-fopenmp", "-fPIC", "-shared", "-o", ORACLE_LIB, src, "-lm"])
    return ORACLE_LIB


def build_reference(verbose=False):
    """Builds oracle/_ref from the reference sources when they are present (no-op otherwise)."""
    script = os.path.join(ORACLE_DIR, "build_ref.sh")
    out = _run(["sh", script])
    if verbose:
        print(out)


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_library(verbose=True, force=force))
    print(build_oracle(verbose=True, force=force))
