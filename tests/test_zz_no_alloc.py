"""zg_run_noalloc, the entry point for callers that cannot allocate device memory while serving
(a memory manager that owns all device memory, or a latency-critical path where cudaMalloc /
cudaFree would synchronise the device).  Called through the C ABI, it must return exactly what
zg_run_async returns for the same query, on two calls in a row that reuse its fixed scratch, under
every record layout, and the device's free memory must not move while it runs.  Collected last
(file name) so that a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

import zgraph as Z

pytestmark = pytest.mark.gpu

NOALLOC_MAX_BLOCKS = 16384  # ZG_NOALLOC_MAX_BLOCKS in include/zgraph_gpu.h


def _counters(prog, dev_buf):
    return prog.result_to_counters(bytes(dev_buf.cpu().numpy()))


@pytest.mark.parametrize("layout", [Z.RECORDS_COMPACT, Z.RECORDS_WIDE, Z.RECORDS_PACKED])
def test_noalloc_matches_async_on_two_calls(layout):
    import torch
    Z.init(0)
    torch.cuda.set_device(0)
    L = Z.lib()
    Z.check(L.zg_set_record_layout(layout))
    try:
        e = Z.gen_rmat(12, 8, seed=21)
        g = Z.Graph.from_edges(e, 1 << 12)
    finally:
        Z.check(L.zg_set_record_layout(Z.RECORDS_AUTO))
    assert g.meta().record_layout == layout
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


def test_noalloc_allocates_nothing():
    """cudaMemGetInfo's free bytes before and after a series of calls (after the first call's
    one-time symbol look-up, with the result buffers already allocated) are equal: no allocation,
    no free, not even one served by a memory pool that would have to grow."""
    import torch
    Z.init(0)
    torch.cuda.set_device(0)
    L = Z.lib()
    g = Z.Graph.from_edges(Z.gen_rmat(13, 8, seed=5), 1 << 13)
    progs = [Z.Program(k) for k in (Z.PROG_TRIANGLE, Z.PROG_FOUR_CLIQUE, Z.PROG_THREE_CHAIN, Z.PROG_FOUR_CHAIN)]
    stream = torch.cuda.current_stream().cuda_stream
    outs = [torch.zeros(112, dtype=torch.uint8, device="cuda") for _ in progs]
    for p, o in zip(progs, outs):  # first calls: the scratch address is looked up once per device
        assert L.zg_run_noalloc(g.handle, p.handle, 1 << 16, 0, 1, 3, C.c_void_p(stream), C.c_void_p(o.data_ptr())) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for rep in range(20):
        for p, o in zip(progs, outs):
            rc = L.zg_run_noalloc(g.handle, p.handle, 1 << 18, rep << 18, 9, 3, C.c_void_p(stream),
                                  C.c_void_p(o.data_ptr()))
            assert rc == 0, L.zg_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_grid_fits_the_scratch():
    """Every program kind and launch variant launches at most 8 resident blocks per SM on compact-
    and packed-record graphs, well within the fixed scratch of ZG_NOALLOC_MAX_BLOCKS blocks (wide-
    record graphs launch up to 24 times that, capped at the scratch size: the noalloc parity test
    above runs one)."""
    import torch
    Z.init(0)
    L = Z.lib()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert 8 * sms <= NOALLOC_MAX_BLOCKS
    for kind in range(Z.PROG_TRIANGLE, Z.PROG_FOUR_CLIQUE_UNBIASED + 1):
        v0, mb, gr = C.c_int(), C.c_int(), C.c_int()
        Z.check(L.zg_get_variant(kind, C.byref(v0), C.byref(mb), C.byref(gr)))
        try:
            for v in range(Z.VARIANTS):
                Z.check(L.zg_set_variant(kind, v))
                Z.check(L.zg_get_variant(kind, C.byref(C.c_int()), C.byref(mb), C.byref(gr)))
                assert 0 < gr.value <= 8 * sms <= NOALLOC_MAX_BLOCKS, (kind, v, gr.value)
        finally:
            Z.check(L.zg_set_variant(kind, v0.value))


def test_noalloc_rejects_null_result():
    Z.init(0)
    L = Z.lib()
    g = Z.Graph.from_edges(np.array([[0, 1], [1, 2], [0, 2]], np.uint32), 3)
    p = Z.Program(Z.PROG_TRIANGLE)
    assert L.zg_run_noalloc(g.handle, p.handle, 10, 0, 1, 0, None, None) == 1
