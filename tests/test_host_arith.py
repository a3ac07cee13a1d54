"""The arithmetic the sampling kernels share with the host, compiled from the library's header by
g++ (tests/host_arith_check.cpp) and checked against Python integers: Philox with per-launch round
keys equals the on-the-fly key schedule; the 192-bit x 32-bit weight multiply is the exact product
(and flags overflow beyond 192 bits); packed edge records give back every field at the widths a
graph may choose; fingerprints stay below the empty entry's field."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        d = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        if os.path.exists(os.path.join(d, "cuda_runtime.h")):
            return d
    return None


@pytest.fixture(scope="module")
def lines(tmp_path_factory):
    inc = _cuda_include()
    if not inc or not shutil.which("g++"):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path_factory.mktemp("arith") / "host_arith_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", inc, "-I", os.path.join(ROOT, "sampling-graph-mining_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "host_arith_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return [ln.split() for ln in out.splitlines()]


def test_philox_round_keys(lines):
    rows = [ln for ln in lines if ln[0] == "philox"]
    assert len(rows) == 64
    for r in rows:
        assert r[5] == r[6], r


def test_weight_multiply_is_exact(lines):
    rows = [ln for ln in lines if ln[0] == "mul"]
    assert len(rows) == 64 and any(r[8] == "1" for r in rows) and any(r[8] == "0" for r in rows)
    for r in rows:
        a = int(r[1]) | int(r[2]) << 64 | int(r[3]) << 128
        p = a * int(r[4])
        got = int(r[5]) | int(r[6]) << 64 | int(r[7]) << 128
        assert got == p % (1 << 192), r
        assert (r[8] == "1") == (p >= 1 << 192), r


def test_packed_fields_round_trip(lines):
    rows = [ln for ln in lines if ln[0] == "packed"]
    assert len(rows) == 6 * 16
    for r in rows:
        assert r[4:10] == r[10:16], r


def test_fingerprint_range(lines):
    (r,) = [ln for ln in lines if ln[0] == "fingerprint_max"]
    assert int(r[1]) < 0x7FFFFFFF
