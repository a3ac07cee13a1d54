"""The multi-GPU path on CPU: two gloo ranks each run their shard of sample indices (here with the
CPU oracle standing in for the device, which returns identical counters) and merge the exact
320-bit sums with zgraph.allgather_counters; the result equals one run over the whole range."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, seed, out_path):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "sampling-graph-mining_gb300"))
    sys.path.insert(0, os.path.join(root, "oracle"))
    import torch.distributed as dist
    import oracle as O
    import zgraph as Z
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    e = Z.gen_rmat(10, 8, seed=3)
    og = O.OracleGraph(e, 1 << 10)
    for kind in (1, 2, 4):
        c = O.run(og, O.OracleProgram(kind), n, seed, kind, first=rank * n, threads=1)
        zc = Z.Counters()
        for f, _ in Z.Counters._fields_:
            setattr(zc, f, getattr(c, f))
        merged = Z.allgather_counters(zc)
        if rank == 0:
            with open(out_path + ".%d" % kind, "w") as f:
                f.write("%d %d %d %s %r\n" % (merged.samples, merged.hits, merged.fails,
                                              " ".join(str(int(x)) for x in merged.sum_num), merged.estimate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_merge_exactly(tmp_path):
    import torch.multiprocessing as mp
    import oracle as O
    import zgraph as Z
    n, seed = 30000, 41
    out = str(tmp_path / "merged")
    mp.start_processes(_worker, args=(2, _free_port(), n, seed, out), nprocs=2, start_method="spawn")
    e = Z.gen_rmat(10, 8, seed=3)
    og = O.OracleGraph(e, 1 << 10)
    for kind in (1, 2, 4):
        whole = O.run(og, O.OracleProgram(kind), 2 * n, seed, kind, first=0)
        got = open(out + ".%d" % kind).read().split()
        assert int(got[0]) == whole.samples and int(got[1]) == whole.hits and int(got[2]) == whole.fails
        assert [int(x) for x in got[3:8]] == [int(x) for x in whole.sum_num]
        assert float(got[8]) == float(whole.exact_sum() / whole.samples)


def test_merge_counters_is_exact():
    import zgraph as Z
    rng = np.random.default_rng(0)
    parts = []
    total = 0
    for _ in range(5):
        c = Z.Counters()
        c.samples = int(rng.integers(1, 1 << 30))
        c.den_log2 = int(rng.integers(0, 3))
        v = int(rng.integers(0, 1 << 62)) << int(rng.integers(0, 120))
        for i in range(5):
            c.sum_num[i] = (v >> (64 * i)) & 0xFFFFFFFFFFFFFFFF
        total += v << (2 - c.den_log2)
        parts.append(c)
    m = Z.merge_counters(parts)
    assert m.den_log2 == 2
    assert sum(int(m.sum_num[i]) << (64 * i) for i in range(5)) == total
