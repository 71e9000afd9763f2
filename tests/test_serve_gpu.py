"""The serving loop (ga_server_*) on the GPU: reads submitted one at a time,
continuous batching with a small in-flight limit so rounds mix reads admitted at
different times, every read's GAF byte-identical to the reference's."""
import os
import sys
import time

import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden_sets import load_gaf, load_graph, load_reads  # noqa: E402

pytestmark = pytest.mark.gpu


def _per_read(gaf: str) -> dict:
    out = {}
    for line in gaf.splitlines(keepends=True):
        out.setdefault(line.split("\t", 1)[0], []).append(line)
    return {k: "".join(v) for k, v in out.items()}


def _serve(aligner, names, seqs, max_in_flight, pause_every=50):
    from graphaligner_gb300.serve import Server
    got = {}
    with Server(aligner, max_reads_in_flight=max_in_flight) as srv:
        name_of = {}
        for i, (n, s) in enumerate(zip(names, seqs)):
            name_of[srv.submit(n, s)] = n
            if i % pause_every == pause_every - 1:
                time.sleep(0.005)
                for r in srv.poll():
                    got[r.ticket] = r
        deadline = time.time() + 300
        while len(got) < len(names) and time.time() < deadline:
            for r in srv.poll(wait_ms=500):
                got[r.ticket] = r
        stats = srv.stats()
    return got, name_of, stats


@pytest.mark.parametrize("graph_name,preset_name,bandwidth,limit", [("vg50k", "vg", 10, 40), ("dbg100k", "dbg", 5, 8)])
def test_served_reads_match_reference(cuda_lib, graph_name, preset_name, bandwidth, limit):
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    g = load_graph(graph_name)
    names, seqs = load_reads(graph_name)
    a = Aligner(Extender(DeviceGraph(g)), g, preset(preset_name, bandwidth=bandwidth))
    got, name_of, stats = _serve(a, names, seqs, limit, pause_every=10)
    assert len(got) == len(names)
    expected = _per_read(load_gaf(graph_name, bandwidth))
    for t, r in got.items():
        assert r.status == 0
        assert r.gaf == expected.get(name_of[t], ""), f"read {name_of[t]} differs"
        assert r.latency_ms >= r.queue_ms >= 0
    assert stats["completed"] == len(names)
    assert stats["max_in_flight"] <= limit
    assert stats["mixed_rounds"] > 0


def test_served_read_alone_equals_in_mix(cuda_lib):
    """A read served alone and the same read served among 199 others give the same bytes."""
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    g = load_graph("vg50k")
    names, seqs = load_reads("vg50k")
    a = Aligner(Extender(DeviceGraph(g)), g, preset("vg"))
    mixed, name_of, _ = _serve(a, names, seqs, 64)
    by_name = {name_of[t]: r.gaf for t, r in mixed.items()}
    for i in (0, 17, 101, 199):
        alone, _, _ = _serve(a, [names[i]], [seqs[i]], 1)
        assert [r.gaf for r in alone.values()] == [by_name[names[i]]]
        assert a.align([names[i]], [seqs[i]]) == by_name[names[i]]
