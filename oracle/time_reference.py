"""Times the reference's own calculate() (oracle/_ref/libzgtime_*.so: its mt19937 Random, its
OpenMP loop) and the oracle port (oracle/zg_oracle.c) on the same graph, threads and sample count:
the check that the port, which bench.py times as the CPU baseline where the reference cannot be
built, runs at the reference's speed.  Test infrastructure; needs oracle/build_ref.sh's output.

  python oracle/time_reference.py [--scale 20] [--edge-factor 3] [--samples 4194304] [--threads N]
"""
import argparse
import ctypes as C
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "sampling-graph-mining_gb300"))
sys.path.insert(0, HERE)
import oracle as O  # noqa: E402
import zgraph as Z  # noqa: E402

APPS = [("triangle", 1), ("four_clique", 2), ("three_chain", 3), ("four_chain", 4)]
# SamplerGenerator patterns (applications/FiveStar.cpp:18-26, FiveHouse.cpp:18-27): program 6
PATTERNS = [("five_star", (5, [(0, 1), (0, 2), (0, 3), (0, 4)])),
            ("five_house", (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)]))]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--edge-factor", type=int, default=3)
    ap.add_argument("--samples", type=int, default=1 << 22)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    e = Z.gen_rmat(args.scale, args.edge_factor, seed=1)
    nv = 1 << args.scale
    edges = np.ascontiguousarray(e, dtype=np.uint32)
    og = O.OracleGraph(edges, nv)
    out = {"graph": "R-MAT scale %d, edge factor %d, %d edges" % (args.scale, args.edge_factor, len(e)),
           "samples": args.samples, "threads": args.threads, "cpu": os.uname().machine, "programs": {}}
    def port_rate(p):
        O.run(og, p, args.samples >> 4, 7, threads=args.threads)  # warm
        t0 = time.perf_counter()
        c = O.run(og, p, args.samples, 11, threads=args.threads)
        return args.samples / (time.perf_counter() - t0), c.estimate

    for name, kind in APPS:
        lib = C.CDLL(os.path.join(HERE, "_ref", "libzgtime_%s.so" % name))
        lib.zgref_time_calculate.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint64, C.c_int,
                                             C.POINTER(C.c_double)]
        lib.zgref_time_calculate.restype = C.c_double
        est = C.c_double(0)
        secs = lib.zgref_time_calculate(edges.ctypes.data, len(e), nv, args.samples, args.threads, C.byref(est))
        rate, pest = port_rate(O.OracleProgram(kind))
        out["programs"][name] = {"reference_samples_per_s": args.samples / secs, "reference_estimate": est.value,
                                 "port_samples_per_s": rate, "port_estimate": pest}
        print(name, out["programs"][name], flush=True)
    lib = C.CDLL(os.path.join(HERE, "_ref", "libzgtime_pattern.so"))
    lib.zgref_time_pattern.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                                       C.c_uint64, C.c_int, C.POINTER(C.c_double)]
    lib.zgref_time_pattern.restype = C.c_double
    for name, (pv, pedges) in PATTERNS:
        pe = np.ascontiguousarray(pedges, dtype=np.uint32)
        est = C.c_double(0)
        secs = lib.zgref_time_pattern(edges.ctypes.data, len(e), nv, pv, len(pe), pe.ctypes.data, args.samples,
                                      args.threads, C.byref(est))
        rate, pest = port_rate(O.OracleProgram(6, pattern=(pv, pedges)))
        out["programs"][name] = {"reference_samples_per_s": args.samples / secs, "reference_estimate": est.value,
                                 "port_samples_per_s": rate, "port_estimate": pest}
        print(name, out["programs"][name], flush=True)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
