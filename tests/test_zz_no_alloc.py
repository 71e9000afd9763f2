"""The allocation-free extension entry point against the regular one.

ga_extend_batch_noalloc is for callers that cannot allocate device memory while
they extend (memory handed out by another allocator under a fixed budget, or
request paths that cannot afford cudaMalloc's device-wide synchronisation).
It keeps all scratch in a fixed device array inside the library, so this test
checks that its results equal ga_extend_batch's on the same batch, on two
calls in a row (the second call sees what the first one left in the array).
The file sorts last so that a run stopping at the first failure has run every
other test first.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_copy(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int8).copy()).cuda()


def test_noalloc_matches_regular_entry_point_twice(cuda_lib):
    torch = pytest.importorskip("torch")
    from graphaligner_gb300 import _abi
    from graphaligner_gb300 import datagen as dg
    from graphaligner_gb300 import graph as gg
    from graphaligner_gb300._lib import check, lib
    from graphaligner_gb300.extend import DeviceGraph, Extender, ExtendParams, pack_batch

    vg = dg.make_variation_graph(20_000, 150, 0.7, 20, seed=21)
    g = gg.build_from_gfa(vg.to_gfa())
    nl = np.zeros(len(vg.node_seqs) + 1, dtype=np.int64)
    nl[1:] = [len(s) for s in vg.node_seqs]
    reads = dg.sample_reads(vg, 40, 22, dg.uniform_length(300, 6000), dg.uniform_error(0.04, 0.15))
    ext = dg.seed_extensions(reads, nl, 15, 23, per_read=2)
    batch = pack_batch(g, ext.seqs, ext.bignode, ext.offset)
    params = ExtendParams(bandwidth=10)

    # the regular entry point (allocates its own buffers)
    dgraph = DeviceGraph(g)
    x = Extender(dgraph)
    expected = x.run(params, batch)

    # the same graph, batch and result buffers in caller-owned device memory
    keep = []

    def dev(a, ctype):
        t = _device_copy(torch, a)
        keep.append(t)
        return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctype))

    u8, u32, u64, i32 = ctypes.c_uint8, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32
    gdesc = _abi.GraphDesc(g.num_nodes, g.first_ambiguous, dev(g.node_length.astype(np.uint32), u32),
                           dev(g.seq2bit.astype(np.uint64), u64), dev(g.seq_ambiguous.astype(np.uint64) if len(g.seq_ambiguous) else np.zeros(1, np.uint64), u64),
                           dev(g.in_offsets.astype(np.uint32), u32), dev(g.in_neighbors.astype(np.uint32), u32),
                           dev(g.out_offsets.astype(np.uint32), u32), dev(g.out_neighbors.astype(np.uint32), u32),
                           dev(g.linearizable.astype(np.uint8), u8), dev(g.component.astype(np.uint32), u32))
    bdesc = _abi.BatchDesc(batch.num, dev(batch.seq, u8), dev(batch.seq_offset, u64), dev(batch.seq_len, u32),
                           dev(batch.start_node, u32), dev(batch.start_offset, u32), dev(batch.trace_offset, u64),
                           dev(batch.trace_capacity, u32))
    n = batch.num
    status = torch.empty(n, dtype=torch.int32, device="cuda")
    score = torch.empty(n, dtype=torch.int32, device="cuda")
    tlen = torch.empty(n, dtype=torch.int32, device="cuda")
    items = torch.empty(batch.total_items, dtype=torch.int64, device="cuda")
    steps = torch.empty(n, dtype=torch.int64, device="cuda")

    def ptr(t, ctype):
        return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctype))

    rdesc = _abi.Results(ptr(status, i32), ptr(score, i32), ptr(tlen, u32), ptr(items, u64), ptr(steps, u64))
    p = params.c()
    stream = torch.cuda.current_stream()
    for call in range(2):
        status.fill_(-7)
        items.fill_(0)
        check(lib().ga_extend_batch_noalloc(ctypes.byref(gdesc), ctypes.byref(p), ctypes.byref(bdesc), ctypes.byref(rdesc),
                                            ctypes.c_void_p(stream.cuda_stream)))
        torch.cuda.synchronize()
        got_status = status.cpu().numpy()
        got_len = tlen.cpu().numpy().view(np.uint32)
        got_items = items.cpu().numpy().view(np.uint64)
        assert np.array_equal(got_status, expected.status), f"call {call}: status differs"
        assert np.array_equal(score.cpu().numpy(), expected.score), f"call {call}: score differs"
        assert np.array_equal(got_len, expected.trace_len), f"call {call}: trace length differs"
        for i in range(n):
            o = int(batch.trace_offset[i])
            assert np.array_equal(got_items[o:o + int(got_len[i])], expected.items(i)), f"call {call}: trace {i} differs"
    x.close()
    dgraph.close()


def test_noalloc_rejects_oversized_batch(cuda_lib):
    torch = pytest.importorskip("torch")
    from graphaligner_gb300 import _abi
    from graphaligner_gb300._lib import lib
    lens = torch.full((4097,), 10, dtype=torch.int32, device="cuda")
    null = ctypes.POINTER(ctypes.c_uint8)()
    gdesc = _abi.GraphDesc()
    bdesc = _abi.BatchDesc()
    bdesc.num = 4097
    bdesc.seq_len = ctypes.cast(ctypes.c_void_p(lens.data_ptr()), ctypes.POINTER(ctypes.c_uint32))
    rdesc = _abi.Results()
    p = _abi.ExtendParams(10, 14705, 2**64 - 1, 294)
    rc = lib().ga_extend_batch_noalloc(ctypes.byref(gdesc), ctypes.byref(p), ctypes.byref(bdesc), ctypes.byref(rdesc), None)
    assert rc != 0
    assert b"4096" in lib().ga_last_error()
    del null


def test_noalloc_rejects_more_than_its_read_bp(cuda_lib):
    """A batch within the extension count but over the 8,000,000 read bp the fixed scratch
    holds is GA_ERR_ARGUMENT with the limit in the message, before any kernel runs (the
    lengths are read back first; the other arrays are never touched)."""
    torch = pytest.importorskip("torch")
    from graphaligner_gb300 import _abi
    from graphaligner_gb300._lib import lib
    n = 2000
    lens = torch.full((n,), 4001, dtype=torch.int32, device="cuda")     # 8,002,000 bp
    dummy = torch.zeros(64, dtype=torch.int64, device="cuda")

    def p(ctype, t=dummy):
        return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctype))

    u8, u32, u64, i32 = ctypes.c_uint8, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32
    gdesc = _abi.GraphDesc(4, 4, p(u32), p(u64), p(u64), p(u32), p(u32), p(u32), p(u32), p(u8), p(u32))
    bdesc = _abi.BatchDesc(n, p(u8), p(u64), p(u32, lens), p(u32), p(u32), p(u64), p(u32))
    rdesc = _abi.Results(p(i32), p(i32), p(u32), p(u64), p(u64))
    params = _abi.ExtendParams(10, 14705, 2**64 - 1, 294)
    rc = lib().ga_extend_batch_noalloc(ctypes.byref(gdesc), ctypes.byref(params), ctypes.byref(bdesc), ctypes.byref(rdesc), None)
    torch.cuda.synchronize()
    assert rc == -1
    assert b"8,000,000" in lib().ga_last_error()
