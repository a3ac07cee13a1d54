"""zg_run_noalloc, the entry point for callers that cannot allocate device memory while serving
(a memory manager that owns all device memory, or a latency-critical path where cudaMalloc /
cudaFree would synchronise the device).  Called through the C ABI, it must return exactly what
zg_run_async returns for the same query, on two calls in a row that reuse its fixed scratch.
Collected last (file name) so that a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

import zgraph as Z

pytestmark = pytest.mark.gpu


def _counters(prog, dev_buf):
    return prog.result_to_counters(bytes(dev_buf.cpu().numpy()))


def test_noalloc_matches_async_on_two_calls():
    import torch
    Z.init(0)
    torch.cuda.set_device(0)
    L = Z.lib()
    e = Z.gen_rmat(12, 8, seed=21)
    g = Z.Graph.from_edges(e, 1 << 12)
    stream = torch.cuda.current_stream().cuda_stream
    n, seed = 1 << 20, 4242
    for kind in (Z.PROG_TRIANGLE, Z.PROG_FOUR_CLIQUE, Z.PROG_FOUR_CHAIN):
        p = Z.Program(kind)
        for call, first in enumerate((0, n)):  # two calls in a row through the shared scratch
            ref = torch.zeros(112, dtype=torch.uint8, device="cuda")
            out = torch.full((112,), 0xAB, dtype=torch.uint8, device="cuda")
            p.run_async(g, n, seed, ref.data_ptr(), stream_id=7, first_sample=first, cuda_stream=stream)
            rc = L.zg_run_noalloc(g.handle, p.handle, n, first, seed, 7, C.c_void_p(stream), C.c_void_p(out.data_ptr()))
            assert rc == 0, L.zg_last_error()
            torch.cuda.synchronize()
            a, b = _counters(p, ref), _counters(p, out)
            assert (b.samples, b.hits, b.fails) == (a.samples, a.hits, a.fails), (kind, call)
            assert [int(x) for x in b.sum_num] == [int(x) for x in a.sum_num], (kind, call)
            assert b.estimate == a.estimate and b.sum_w == a.sum_w and b.sum_w2 == a.sum_w2, (kind, call)
            assert b.samples == n


def test_noalloc_rejects_null_result():
    Z.init(0)
    L = Z.lib()
    g = Z.Graph.from_edges(np.array([[0, 1], [1, 2], [0, 2]], np.uint32), 3)
    p = Z.Program(Z.PROG_TRIANGLE)
    assert L.zg_run_noalloc(g.handle, p.handle, 10, 0, 1, 0, None, None) == 1
