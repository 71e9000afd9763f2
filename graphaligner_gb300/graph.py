"""Host-side alignment graph: the AlignmentGraph fields the DP reads, as arrays.

Two sources:

* ``load_gag`` reads the GAG1 binary layout (arrays of an AlignmentGraph built by
  GraphAligner's own ``DirectedGraph::BuildFromGFA`` + ``AlignmentGraph::Finalize``,
  dumped field by field), so the GPU path runs on the reference's exact node
  numbering, component order and neighbour order.
* ``build_from_gfa`` builds the same kind of graph from a GFA with 0-bp overlaps
  (the variation-graph workloads) or constant k-1 overlaps (de Bruijn graphs), in
  native code (csrc/gfa_build.cpp).  It follows AlignmentGraph's construction
  rules (AlignmentGraph.cpp:48-296): both strands (GFA id*2 forward, id*2+1
  reverse complement), nodes split into pieces of at most 64 bp, ambiguous
  nodes renumbered to the end, the linearizable flags of findLinearizable, the
  Tarjan component order of doComponentOrder and the chains of findChains.  Its
  node numbering is its own (GFA order); results are exact against the oracle on
  the same arrays.
"""
from __future__ import annotations

import ctypes
import dataclasses
import numpy as np

SPLIT_NODE_SIZE = 64

@dataclasses.dataclass
class Graph:
    num_nodes: int
    first_ambiguous: int
    node_length: np.ndarray      # uint32 [N]
    node_ids: np.ndarray         # int32  [N] bigraph node id (GFA id*2 + strand)
    node_offset: np.ndarray      # uint32 [N] offset of the piece inside its bigraph node
    reverse: np.ndarray          # uint8  [N]
    linearizable: np.ndarray     # uint8  [N]
    component: np.ndarray        # uint32 [N]
    chain_number: np.ndarray     # uint64 [N]
    chain_approx_pos: np.ndarray # uint64 [N]
    seq2bit: np.ndarray          # uint64 [first_ambiguous * 2]
    seq_ambiguous: np.ndarray    # uint64 [(N - first_ambiguous) * 4] A,C,G,T
    in_offsets: np.ndarray       # uint32 [N + 1]
    in_neighbors: np.ndarray     # uint32
    out_offsets: np.ndarray      # uint32 [N + 1]
    out_neighbors: np.ndarray    # uint32
    lookup_ids: np.ndarray       # int32  [M] bigraph node ids in nodeLookup order
    original_size: np.ndarray    # uint32 [M]
    lookup_offsets: np.ndarray   # uint32 [M + 1]
    lookup_nodes: np.ndarray     # uint32 split nodes of each bigraph node, in offset order
    names: list                  # [M] original names ("" = numeric GFA id)
    bp_size: int = 0

    def __post_init__(self):
        self._lookup_index = {int(b): i for i, b in enumerate(self.lookup_ids)}

    # AlignmentGraph::GetUnitigNode (AlignmentGraph.cpp:812-828)
    def unitig_node(self, bignode: int, offset: int) -> tuple[int, int]:
        i = self._lookup_index[int(bignode)]
        nodes = self.lookup_nodes[self.lookup_offsets[i]:self.lookup_offsets[i + 1]]
        starts = self.node_offset[nodes]
        k = int(np.searchsorted(starts, offset, side="right")) - 1
        node = int(nodes[k])
        return node, int(offset - self.node_offset[node])

    def original_size_of(self, bignode: int) -> int:
        return int(self.original_size[self._lookup_index[int(bignode)]])

    # AlignmentGraph::GetReversePosition (AlignmentGraph.cpp:830-847)
    def reverse_position(self, bignode: int, offset: int) -> tuple[int, int]:
        size = self.original_size_of(bignode)
        return (bignode ^ 1), size - offset - 1

    def node_sequence(self, node: int) -> str:
        n = int(self.node_length[node])
        if node < self.first_ambiguous:
            w = self.seq2bit[node * 2:node * 2 + 2]
            return "".join("ACGT"[(int(w[p // 32]) >> ((p % 32) * 2)) & 3] for p in range(n))
        a = self.seq_ambiguous[(node - self.first_ambiguous) * 4:(node - self.first_ambiguous) * 4 + 4]
        table = "?ACMGRSVTWYHKDBN"
        return "".join(table[sum(((int(a[c]) >> p) & 1) << c for c in range(4))] for p in range(n))

    def char_table(self) -> np.ndarray:
        """[N, 64] uint8 characters of every split node (AlignmentGraph::NodeSequences)."""
        out = np.zeros((self.num_nodes, 64), dtype=np.uint8)
        fa = self.first_ambiguous
        if fa:
            w = self.seq2bit.reshape(fa, 2)
            pos = np.arange(64)
            codes = (w[:, pos // 32] >> (2 * (pos % 32)).astype(np.uint64)) & np.uint64(3)
            out[:fa] = np.frombuffer(b"ACGT", dtype=np.uint8)[codes.astype(np.int64)]
        for n in range(fa, self.num_nodes):
            s = self.node_sequence(n).encode()
            out[n, :len(s)] = np.frombuffer(s, dtype=np.uint8)
        return out

    def desc(self):
        """A ga_graph_desc ctypes struct pointing at this graph's arrays."""
        from ._abi import GraphDesc
        return GraphDesc.from_graph(self)


def _arr(buf, off, dtype, count):
    n = np.dtype(dtype).itemsize * count
    return np.frombuffer(buf, dtype=dtype, count=count, offset=off).copy(), off + n


def load_gag(path: str) -> Graph:
    """Reads the GAG1 layout written by the reference-graph dumper."""
    buf = open(path, "rb").read()
    if buf[:4] != b"GAG1":
        raise ValueError(f"{path}: not a GAG1 graph")
    hdr = np.frombuffer(buf, dtype=np.uint64, count=8, offset=4)
    N, fa, n_in, n_out, M, n_lookup, n_names, bp = (int(x) for x in hdr)
    off = 4 + 64
    node_length, off = _arr(buf, off, np.uint32, N)
    node_ids, off = _arr(buf, off, np.int32, N)
    node_offset, off = _arr(buf, off, np.uint32, N)
    reverse, off = _arr(buf, off, np.uint8, N)
    linearizable, off = _arr(buf, off, np.uint8, N)
    component, off = _arr(buf, off, np.uint32, N)
    chain_number, off = _arr(buf, off, np.uint64, N)
    chain_pos, off = _arr(buf, off, np.uint64, N)
    seq2, off = _arr(buf, off, np.uint64, fa * 2)
    seqa, off = _arr(buf, off, np.uint64, (N - fa) * 4)
    in_off, off = _arr(buf, off, np.uint32, N + 1)
    in_nb, off = _arr(buf, off, np.uint32, n_in)
    out_off, off = _arr(buf, off, np.uint32, N + 1)
    out_nb, off = _arr(buf, off, np.uint32, n_out)
    lookup_ids, off = _arr(buf, off, np.int32, M)
    orig_size, off = _arr(buf, off, np.uint32, M)
    lookup_off, off = _arr(buf, off, np.uint32, M + 1)
    lookup_nodes, off = _arr(buf, off, np.uint32, n_lookup)
    name_len, off = _arr(buf, off, np.uint32, M)
    blob = buf[off:off + n_names].decode()
    names, p = [], 0
    for ln in name_len:
        names.append(blob[p:p + int(ln)])
        p += int(ln)
    return Graph(N, fa, node_length, node_ids, node_offset, reverse, linearizable, component,
                 chain_number, chain_pos, seq2, seqa, in_off, in_nb, out_off, out_nb,
                 lookup_ids, orig_size, lookup_off, lookup_nodes, names, bp)


def save_gag(g: Graph, path: str) -> None:
    with open(path, "wb") as f:
        f.write(b"GAG1")
        blob = "".join(g.names).encode()
        f.write(np.array([g.num_nodes, g.first_ambiguous, len(g.in_neighbors), len(g.out_neighbors),
                          len(g.lookup_ids), len(g.lookup_nodes), len(blob), g.bp_size], dtype=np.uint64).tobytes())
        for a, dt in ((g.node_length, np.uint32), (g.node_ids, np.int32), (g.node_offset, np.uint32),
                      (g.reverse, np.uint8), (g.linearizable, np.uint8), (g.component, np.uint32),
                      (g.chain_number, np.uint64), (g.chain_approx_pos, np.uint64), (g.seq2bit, np.uint64),
                      (g.seq_ambiguous, np.uint64), (g.in_offsets, np.uint32), (g.in_neighbors, np.uint32),
                      (g.out_offsets, np.uint32), (g.out_neighbors, np.uint32), (g.lookup_ids, np.int32),
                      (g.original_size, np.uint32), (g.lookup_offsets, np.uint32), (g.lookup_nodes, np.uint32),
                      (np.array([len(n.encode()) for n in g.names], dtype=np.uint32), np.uint32)):
            f.write(np.ascontiguousarray(a, dtype=dt).tobytes())
        f.write(blob)


class _GfaArrays(ctypes.Structure):
    """ga_gfa_graph_arrays (csrc/gfa_build.h)."""
    _fields_ = [
        ("num_nodes", ctypes.c_uint32),
        ("first_ambiguous", ctypes.c_uint32),
        ("num_lookup", ctypes.c_uint32),
        ("num_in_edges", ctypes.c_uint64),
        ("num_out_edges", ctypes.c_uint64),
        ("num_lookup_nodes", ctypes.c_uint64),
        ("bp_size", ctypes.c_uint64),
    ] + [(name, ctypes.c_void_p) for name in (
        "node_length", "node_ids", "node_offset", "reverse", "linearizable", "component", "chain_number",
        "chain_approx_pos", "seq2bit", "seq_ambiguous", "in_offsets", "in_neighbors", "out_offsets",
        "out_neighbors", "lookup_ids", "original_size", "lookup_offsets", "lookup_nodes", "names")] + [
        ("names_bytes", ctypes.c_uint64),
    ]


def build_from_gfa(gfa_text: str) -> Graph:
    """Alignment graph from a GFA (0-bp overlaps or de Bruijn k-1 overlaps).

    An overlap of ``o`` bp on a link enters the target strand at offset ``o``: both
    strands get a breakpoint there, pieces are cut between breakpoints in 64-bp steps
    from each breakpoint, and the link joins the source's last piece to the target's
    piece that starts at ``o`` (DirectedGraph::BuildFromGFA, BigraphToDigraph.cpp:214-266;
    AlignmentGraph::AddNode / AddEdgeNodeId, AlignmentGraph.cpp:47-80, 230-248).
    Raises GAError for a GFA it cannot take (unknown segment in a link, an overlap not
    smaller than both segments, an empty segment, a non-IUPAC character)."""
    from .build import build
    from ._lib import check, lib
    build()
    data = gfa_text.encode()
    handle = ctypes.c_void_p()
    a = _GfaArrays()
    check(lib().ga_gfa_build(data, ctypes.c_uint64(len(data)), ctypes.byref(handle), ctypes.byref(a)))
    try:
        def take(name, count, dtype):
            if count == 0:
                return np.zeros(0, dtype=dtype)
            buf = (ctypes.c_uint8 * (int(count) * np.dtype(dtype).itemsize)).from_address(getattr(a, name))
            return np.frombuffer(buf, dtype=dtype).copy()
        n, fa, m = a.num_nodes, a.first_ambiguous, a.num_lookup
        names = ctypes.string_at(a.names, a.names_bytes).split(b"\0")[:m] if a.names_bytes else []
        return Graph(n, fa, take("node_length", n, np.uint32), take("node_ids", n, np.int32),
                     take("node_offset", n, np.uint32), take("reverse", n, np.uint8),
                     take("linearizable", n, np.uint8), take("component", n, np.uint32),
                     take("chain_number", n, np.uint64), take("chain_approx_pos", n, np.uint64),
                     take("seq2bit", fa * 2, np.uint64), take("seq_ambiguous", (n - fa) * 4, np.uint64),
                     take("in_offsets", n + 1, np.uint32), take("in_neighbors", a.num_in_edges, np.uint32),
                     take("out_offsets", n + 1, np.uint32), take("out_neighbors", a.num_out_edges, np.uint32),
                     take("lookup_ids", m, np.int32), take("original_size", m, np.uint32),
                     take("lookup_offsets", m + 1, np.uint32), take("lookup_nodes", a.num_lookup_nodes, np.uint32),
                     [x.decode() for x in names], int(a.bp_size))
    finally:
        lib().ga_gfa_free(handle)
