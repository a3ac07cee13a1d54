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


CPP = os.path.join(PKG, "cpp")
HOST_LIB = os.path.join(BUILD, "libzgraph_host.so")
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function", "-I" + os.path.join(CPP, "include")]


def _cxx():
    return os.environ.get("CXX", "g++")


def build_host(verbose=False, force=False):
    """libzgraph_host.so: the C++ host layer (the reference's class interface over the C ABI)."""
    lib = build_library(verbose=verbose, force=force)
    src_dir = os.path.join(CPP, "src")
    inc_dir = os.path.join(CPP, "include")
    headers = [os.path.join(inc_dir, f) for f in os.listdir(inc_dir)] + \
              [os.path.join(src_dir, f) for f in os.listdir(src_dir) if f.endswith(".hpp")] + \
              [os.path.join(ROOT, "include", "zgraph_gpu.h")]
    units = sorted(f for f in os.listdir(src_dir) if f.endswith(".cpp"))
    objs, jobs = [], []
    for u in units:
        src = os.path.join(src_dir, u)
        obj = os.path.join(BUILD, "host_" + u + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([_cxx()] + CXX_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or _stale(HOST_LIB, objs + [lib]):
        _run([_cxx(), "-shared", "-o", HOST_LIB] + objs +
             ["-L" + BUILD, "-lzgraph_gpu", "-Wl,-rpath,$ORIGIN"])
    return HOST_LIB


def build_app(sources, out, include_dirs=(), extra_flags=()):
    """Compiles an application written against the reference's headers and links it to the host
    layer; the executable finds both libraries through its rpath."""
    build_host()
    cmd = [_cxx()] + CXX_FLAGS + ["-I" + d for d in include_dirs] + list(extra_flags) + list(sources) + \
          ["-o", out, "-L" + BUILD, "-lzgraph_host", "-lzgraph_gpu", "-Wl,-rpath," + BUILD, "-lpthread"]
    _run(cmd)
    return out


def build_oracle(verbose=False, force=False):
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    srcs = [os.path.join(ORACLE_DIR, f) for f in ("zg_oracle.c", "zgo_gen.c")]
    deps = srcs + [os.path.join(ORACLE_DIR, "zg_oracle.h"), os.path.join(ROOT, "include", "zgraph_gpu.h")]
    if force or _stale(ORACLE_LIB, deps):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O2", "-fopenmp", "-fPIC", "-shared", "-o", ORACLE_LIB] + srcs + ["-lm"])
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
