"""The C-ABI library loads without a GPU and exports every entry point include/zgraph_gpu.h declares;
the binding's struct layouts match the header; host-only entry points work without a device."""
import ctypes
import os
import re

import numpy as np

import zgraph as Z
from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "zgraph_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(zg_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    L = Z.lib()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_struct_layouts():
    assert ctypes.sizeof(Z.Counters) == 8 * 3 + 4 * 2 + 8 * 5 + 8 * 4
    assert Z.TRACE_DTYPE.itemsize == 4 * 6 + 8 + 8 * 3 + 8 * 16 * 3
    assert ctypes.sizeof(Z.GraphMeta) == 4 * 2 + 8 * 4 + 4 * 2


def test_version_and_errors_without_device():
    L = Z.lib()
    assert L.zg_version() >= 1
    # null arguments are rejected with a status code, never a crash
    assert L.zg_graph_create(None, 5, 4, None, None, None) == 1
    assert L.zg_program_create(99, 0, ctypes.byref(ctypes.c_void_p())) == 5
    assert b"unknown program kind" in L.zg_last_error()


def test_result_conversion_is_exact():
    """zg_result_to_counters: carry-saved 32-bit lanes -> 320-bit sum -> mean rounded once."""
    from fractions import Fraction
    import struct
    rng = np.random.default_rng(3)
    p = Z.Program(Z.PROG_FOUR_CLIQUE)  # den_log2 = 2; no device memory needed
    for trial in range(300):
        n = int(rng.integers(1, 1 << 40))
        bits = int(rng.integers(1, 50))
        lanes = [int(x) for x in rng.integers(0, 1 << bits, size=8, dtype=np.uint64)]
        if trial % 3 == 0:
            lanes = [0] * 7 + [int(rng.integers(0, 4))]
        blob = struct.pack("<4Q8Q2d", n, 5, 1, 0, *lanes, 1.5, 2.5)
        c = p.result_to_counters(blob)
        total = sum(v << (32 * i) for i, v in enumerate(lanes))
        assert sum(int(c.sum_num[i]) << (64 * i) for i in range(5)) == total
        assert c.estimate == float(Fraction(total, 4 * n))
        assert (c.samples, c.hits, c.fails, c.sum_w2) == (n, 5, 1, 2.5)
        assert c.sum_w == float(Fraction(total, 4))  # the exact sum, rounded once


def test_generators_are_deterministic_and_simple():
    a = Z.gen_rmat(12, 8, seed=1)
    b = Z.gen_rmat(12, 8, seed=1)
    c = Z.gen_rmat(12, 8, seed=2)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    for e in (a, Z.gen_chung_lu(5000, 2.3, 10.0, seed=3)):
        assert np.all(e[:, 0] != e[:, 1])
        key = np.minimum(e[:, 0], e[:, 1]).astype(np.uint64) << np.uint64(32) | np.maximum(e[:, 0], e[:, 1])
        assert len(np.unique(key)) == len(e)
    w = Z.gen_weights(10000, 100, seed=4)
    assert w.min() >= 0 and w.max() < 100 and len(np.unique(w)) == 100
    # R-MAT scale 13, edge factor 12 (the reference's CPU-runnable workload): ~80K edges
    assert 70000 < len(Z.gen_rmat(13, 12, seed=1)) < 100000


def _prototypes():
    """Every zg_* prototype of include/zgraph_gpu.h: name -> (return type, [parameter types])."""
    text = open(os.path.join(ROOT, "include", "zgraph_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"^\s*#.*$", "", text, flags=re.M)
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(zg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        ret, name, params = " ".join(m.group(1).split()), m.group(2), m.group(3).strip()
        types = [] if params in ("", "void") else [re.sub(r"\b\w+\s*(\[\d*\])?$", lambda t: "*" if t.group(1) else "",
                                                          p.strip()).strip() for p in params.split(",")]
        protos[name] = (ret, types)
    return protos


def _c_kind(t):
    """A C type as the ABI sees it: ('p',) pointer, ('f', bits) floating, ('i', bits, signed)."""
    t = " ".join(t.replace("const", "").split())
    if "*" in t:
        return ("p",)
    if t in ("double", "float"):
        return ("f", 64 if t == "double" else 32)
    width = {"int": 32, "int32_t": 32, "uint32_t": 32, "int64_t": 64, "uint64_t": 64}[t]
    return ("i", width, not t.startswith("u"))


def _ctypes_kind(ct):
    if ct is ctypes.c_char_p or ct is ctypes.c_void_p or (isinstance(ct, type) and issubclass(ct, ctypes._Pointer)):
        return ("p",)
    if ct in (ctypes.c_double, ctypes.c_float):
        return ("f", 8 * ctypes.sizeof(ct))
    signed = ct in (ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.c_long, ctypes.c_longlong)
    return ("i", 8 * ctypes.sizeof(ct), signed)


def test_binding_signatures_match_the_header():
    """The ctypes binding (zgraph.lib()) declares every entry point with the header's parameter
    count, and each parameter and return value with the same kind: pointer, floating point of the
    same width, or integer of the same width and signedness.  A mismatch would pass arguments in the
    wrong registers or truncate them without any error."""
    L = Z.lib()
    protos = _prototypes()
    assert set(protos) == set(declared_symbols())
    bound = [n for n in protos if getattr(L, n).argtypes is not None]
    assert len(bound) >= len(protos) - 2, sorted(set(protos) - set(bound))
    bad = []
    for name in bound:
        ret, params = protos[name]
        f = getattr(L, name)
        if len(f.argtypes) != len(params):
            bad.append((name, "arity", len(f.argtypes), len(params)))
            continue
        for i, (ct, p) in enumerate(zip(f.argtypes, params)):
            if _ctypes_kind(ct) != _c_kind(p):
                bad.append((name, i, p, ct))
        want = _c_kind(ret)
        got = _ctypes_kind(f.restype)
        if want != got:
            bad.append((name, "return", ret, f.restype))
    assert not bad, bad
