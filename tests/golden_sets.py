"""Loads the golden vectors in tests/golden/ (made by tests/golden/make_golden.py
from the reference's own source) and digests results in the same form."""
from __future__ import annotations

import gzip
import hashlib
import os
import tempfile

import numpy as np

from graphaligner_gb300 import graph as gg
from graphaligner_gb300.extend import pack_batch

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


GRAPH_OF = {"vg50k_hi": "vg50k", "vg50k_px": "vg50k"}
# tangle effort (maxCellsPerSlice) the extension digests were made with; unlimited otherwise
MAX_CELLS = {"dbg100k": 10000, "dbg1m": 10000}
# X-drop cutoffs with digests of their own (at the set's first bandwidth); the default otherwise
XDROPS = {"vg50k_px": (1500, 3000)}


def load_graph(name: str):
    name = GRAPH_OF.get(name, name)
    with tempfile.NamedTemporaryFile(suffix=".gag") as f:
        f.write(gzip.open(os.path.join(GOLDEN, f"{name}_graph.gag.gz")).read())
        f.flush()
        return gg.load_gag(f.name)


def load_requests(name: str):
    seqs, nodes, offs = [], [], []
    for line in gzip.open(os.path.join(GOLDEN, f"{name}_ext.tsv.gz"), "rt"):
        a, b, c = line.rstrip("\n").split("\t")
        nodes.append(int(a))
        offs.append(int(b))
        seqs.append(c.encode())
    return seqs, np.array(nodes), np.array(offs)


def load_digests(name: str, bandwidth: int, xdrop: int | None = None):
    """(status, score, items, sha1) per request of the set, from the reference at this
    bandwidth and, when given, X-drop cutoff."""
    out = []
    suffix = f"_x{xdrop}" if xdrop is not None else ""
    for line in open(os.path.join(GOLDEN, f"{name}_ext_b{bandwidth}{suffix}.digest")):
        s, sc, n, h = line.split()
        out.append((int(s), int(sc), int(n), h))
    return out


def digest(result, i: int):
    status = int(result.status[i])
    if status != 0:
        return (status, 0, 0, hashlib.sha1(b"").hexdigest())
    items = np.ascontiguousarray(result.items(i))
    return (status, int(result.score[i]), len(items), hashlib.sha1(items.tobytes()).hexdigest())


def golden_case(name: str):
    g = load_graph(name)
    seqs, nodes, offs = load_requests(name)
    return g, pack_batch(g, seqs, nodes, offs)


def compare(result, expected):
    """Indices whose (status, score, n, digest) differ."""
    bad = []
    for i, e in enumerate(expected):
        d = digest(result, i)
        if e[0] != 0:
            if d[0] != e[0]:
                bad.append(i)
        elif d != e:
            bad.append(i)
    return bad


def load_reads(name: str = "vg50k"):
    names, seqs = [], []
    for line in gzip.open(os.path.join(GOLDEN, f"{name}_reads.fa.gz"), "rt"):
        line = line.rstrip("\n")
        if line.startswith(">"):
            names.append(line[1:].split()[0])
            seqs.append("")
        elif line:
            seqs[-1] += line
    return names, [s.encode() for s in seqs]


def load_gaf(name: str, bandwidth: int) -> str:
    return gzip.open(os.path.join(GOLDEN, f"{name}_b{bandwidth}.gaf.gz"), "rt").read()


def graph_file(name: str, directory: str) -> str:
    """Writes the golden graph as a plain GAG1 file into directory and returns its path."""
    name = GRAPH_OF.get(name, name)
    path = os.path.join(directory, f"{name}.gag")
    open(path, "wb").write(gzip.open(os.path.join(GOLDEN, f"{name}_graph.gag.gz")).read())
    return path
