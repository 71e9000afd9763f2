"""Python restatement of the package's GFA builder (graph.build_from_gfa, built natively in
graphaligner_gb300/csrc/gfa_build.cpp): the same construction rules step for step, kept as
the checker the native builder is compared with array by array (tests/test_graph_build.py).
It follows DirectedGraph::BuildFromGFA (BigraphToDigraph.cpp:214-266) and AlignmentGraph's
construction and Finalize (AlignmentGraph.cpp:47-80, 230-248, 300-724, 898-1094)."""
from __future__ import annotations

import numpy as np

from graphaligner_gb300.graph import SPLIT_NODE_SIZE, Graph

_CODE = np.full(256, 255, dtype=np.uint8)
for _i, _c in enumerate(b"ACGT"):
    _CODE[_c] = _i
    _CODE[ord(chr(_c).lower())] = _i
_CODE[ord("U")] = 3
_CODE[ord("u")] = 3
_IUPAC = {
    "A": 1, "C": 2, "G": 4, "T": 8, "U": 8, "R": 5, "Y": 10, "K": 12, "M": 3,
    "S": 6, "W": 9, "B": 14, "D": 13, "H": 11, "V": 7, "N": 15,
}
_COMPLEMENT = bytes.maketrans(b"ACGTUacgtuRYKMSWBDHVNrykmswbdhvn", b"TGCAAtgcaaYRMKSWVHDBNyrmkswvhdbn")


def _csr(lists):
    off = np.zeros(len(lists) + 1, dtype=np.uint32)
    off[1:] = np.cumsum([len(x) for x in lists])
    flat = np.fromiter((v for x in lists for v in x), dtype=np.uint32, count=int(off[-1]))
    return off, flat


def _find_linearizable(in_lists):
    """AlignmentGraph::findLinearizable (AlignmentGraph.cpp:632-724), step for step.

    The reference marks a node checked before pushing it, and its walk ends as
    soon as the top of the stack is checked, so every walk ends on its first
    step and no node is ever marked linearizable.  The restatement keeps that
    behaviour (the flag feeds the queue-seeding skip at
    GraphAlignerBitvectorBanded.h:317)."""
    n = len(in_lists)
    lin = np.zeros(n, dtype=np.uint8)
    checked = np.zeros(n, dtype=bool)
    on_stack = np.zeros(n, dtype=bool)
    for node in range(n):
        if checked[node]:
            continue
        if len(in_lists[node]) != 1:
            checked[node] = True
            continue
        checked[node] = True
        stack = [node]
        on_stack[node] = True
        while True:
            top = stack[-1]
            if len(in_lists[top]) != 1 or checked[top]:
                for s_ in stack[:-1]:
                    checked[s_] = True
                    lin[s_] = 1
                    on_stack[s_] = False
                lin[top] = 0
                checked[top] = True
                on_stack[top] = False
                break
            nb = in_lists[top][0]
            if nb == node:
                for s_ in stack:
                    checked[s_] = True
                    lin[s_] = 0
                    on_stack[s_] = False
                break
            if on_stack[nb]:
                k = stack.index(nb)
                for s_ in stack[k + 1:]:
                    checked[s_] = True
                    lin[s_] = 0
                    on_stack[s_] = False
                for s_ in stack[:k]:
                    checked[s_] = True
                    lin[s_] = 1
                    on_stack[s_] = False
                break
            stack.append(nb)
            on_stack[nb] = True
    return lin


def _component_order(out_lists):
    """AlignmentGraph::doComponentOrder (AlignmentGraph.cpp:987-1094): iterative Tarjan
    from node 0 upward, components numbered in reverse finishing order so that every
    edge goes from a lower to an equal or higher component number."""
    n = len(out_lists)
    UNSET = -1
    index = np.full(n, UNSET, dtype=np.int64)
    low = np.full(n, UNSET, dtype=np.int64)
    on_stack = np.zeros(n, dtype=bool)
    comp = np.full(n, UNSET, dtype=np.int64)
    stack = []
    counter = 0
    next_comp = 0
    for root in range(n):
        if index[root] != UNSET:
            continue
        call = [(root, 0)]
        index[root] = low[root] = counter
        counter += 1
        stack.append(root)
        on_stack[root] = True
        while call:
            v, i = call[-1]
            outs = out_lists[v]
            if i < len(outs):
                w = outs[i]
                call[-1] = (v, i + 1)
                if index[w] == UNSET:
                    index[w] = low[w] = counter
                    counter += 1
                    stack.append(w)
                    on_stack[w] = True
                    call.append((w, 0))
                elif on_stack[w]:
                    low[v] = min(low[v], index[w])
                continue
            call.pop()
            if call:
                u = call[-1][0]
                low[u] = min(low[u], low[v])
            if low[v] == index[v]:
                while True:
                    w = stack.pop()
                    on_stack[w] = False
                    comp[w] = next_comp
                    if w == v:
                        break
                next_comp += 1
    return (next_comp - 1 - comp).astype(np.uint32)


def _find_chains(n, in_lists, out_lists, comp, lookup_pieces, node_length):
    """AlignmentGraph::findChains (AlignmentGraph.cpp:571-630) with chainTips (428-519),
    chainCycles (521-569), chainBubble / findBubble (300-393) and fixChainApproxPos
    (395-426): union-find with union by rank (merge, AlignmentGraph.cpp:344-354,
    including its rank bump when both sides already share a root), bigraph nodes
    visited in nodeLookup order."""
    parent = list(range(n))
    rank = [0] * n
    max_ = (1 << 64) - 1

    def find(x):
        root = x
        while parent[root] != root:
            root = parent[root]
        while parent[x] != root:
            parent[x], x = root, parent[x]
        return root

    def merge(a, b):
        a, b = find(a), find(b)
        if rank[a] < rank[b]:
            a, b = b, a
        parent[b] = a
        if rank[a] == rank[b]:
            rank[a] += 1

    for pieces in lookup_pieces:
        for k in range(1, len(pieces)):
            merge(pieces[0], pieces[k])
    # chainTips
    ignorable = [False] * n
    order = sorted(range(n), key=lambda i: comp[i])
    ncomp = int(comp[order[-1]]) + 1 if n else 0
    fw = [True] * ncomp
    for i in reversed(order):
        ci = comp[i]
        if not fw[ci]:
            continue
        for nb in out_lists[i]:
            if comp[nb] == ci or not fw[comp[nb]]:
                fw[ci] = False
                break
    for i in reversed(order):
        if fw[comp[i]]:
            for nb in out_lists[i]:
                merge(i, nb)
    bw = [True] * ncomp
    for i in order:
        ci = comp[i]
        if not bw[ci]:
            continue
        for nb in in_lists[i]:
            if comp[nb] == ci or not bw[comp[nb]]:
                bw[ci] = False
                break
    for i in order:
        if bw[comp[i]]:
            for nb in in_lists[i]:
                merge(i, nb)
    tip_chainers = {}
    for i in range(n):
        b_, f_ = bw[comp[i]], fw[comp[i]]
        if b_ or f_:
            ignorable[i] = True
        # the reference compares raw parent entries here, not roots
        if b_:
            for nb in out_lists[i]:
                if parent[nb] != parent[i]:
                    tip_chainers.setdefault(parent[i], []).append(nb)
        if f_:
            for nb in in_lists[i]:
                if parent[nb] != parent[i]:
                    tip_chainers.setdefault(parent[i], []).append(nb)
    # chainCycles
    for i in range(n):
        ufw = max_
        for u in out_lists[i]:
            if ignorable[u] or u == i:
                continue
            ufw = u if ufw == max_ else max_ - 1
        ubw = max_
        for u in in_lists[i]:
            if ignorable[u] or u == i:
                continue
            if ubw == max_:
                ubw = u
            elif u != ubw:
                ubw = max_ - 1
        if ufw != ubw or ufw >= max_ - 1:
            continue
        ignorable[i] = True
        merge(i, ufw)

    # chainBubble from the last piece of every bigraph node
    def find_bubble(start):
        stack = [start]
        visited = set()
        seen = {start}
        while stack:
            v = stack.pop()
            seen.discard(v)
            visited.add(v)
            if not out_lists[v]:
                return None
            for u in out_lists[v]:
                if ignorable[u] or u == v:
                    continue
                if u == start:
                    return None
                seen.add(u)
                if not any((w != u and not ignorable[w] and w not in visited) for w in in_lists[u]):
                    stack.append(u)
            if len(stack) == 1 and len(seen) == 1 and stack[0] in seen:
                t = stack[-1]
                if start in out_lists[t]:
                    return None
                return t
        return None

    for pieces in lookup_pieces:
        start = pieces[-1]
        end = find_bubble(start)
        if end is None:
            continue
        merge(start, end)
        visited = set()
        stack = [start]
        while stack:
            top = stack.pop()
            if top in visited or ignorable[top]:
                continue
            visited.add(top)
            merge(start, top)
            for nb in out_lists[top]:
                if nb not in visited and nb != end:
                    stack.append(nb)
    for key, nbs in tip_chainers.items():
        if len({parent[x] for x in nbs}) != 1:
            continue
        merge(key, nbs[0])
    chain = np.array([find(i) for i in range(n)], dtype=np.uint64)
    # fixChainApproxPos
    pos = np.full(n, max_, dtype=np.uint64)
    big = (n + 5) * SPLIT_NODE_SIZE
    for s0 in range(n):
        if pos[s0] != max_:
            continue
        c = chain[s0]
        stack = [(s0, big)]
        while stack:
            v, d = stack.pop()
            if pos[v] != max_:
                continue
            pos[v] = d
            for u in out_lists[v]:
                if chain[u] == c and pos[u] == max_:
                    stack.append((u, d + int(node_length[u])))
            for u in in_lists[v]:
                if chain[u] == c and pos[u] == max_:
                    stack.append((u, d - int(node_length[v])))
    return chain, pos


def build_from_gfa(gfa_text: str) -> Graph:
    """Alignment graph from a GFA (0-bp overlaps or de Bruijn k-1 overlaps).

    An overlap of ``o`` bp on a link enters the target strand at offset ``o``: both
    strands get a breakpoint there, pieces are cut between breakpoints in 64-bp steps
    from each breakpoint, and the link joins the source's last piece to the target's
    piece that starts at ``o`` (DirectedGraph::BuildFromGFA, BigraphToDigraph.cpp:214-266;
    AlignmentGraph::AddNode / AddEdgeNodeId, AlignmentGraph.cpp:47-80, 230-248)."""
    seqs = {}
    order = []
    links = []
    for line in gfa_text.splitlines():
        if not line or line[0] not in "SL":
            continue
        f = line.split("\t")
        if f[0] == "S":
            seqs[f[1]] = f[2]
            order.append(f[1])
        else:
            ov = 0 if f[5] == "*" else int(f[5].rstrip("MS"))
            links.append((f[1], f[2] == "+", f[3], f[4] == "+", ov))
    numeric = all(s.lstrip("-").isdigit() for s in order)
    ids = {name: (int(name) if numeric else k + 1) for k, name in enumerate(order)}
    breaks = {}
    for a, ap, b, bp, ov in links:
        if ov >= len(seqs[a]) or ov >= len(seqs[b]):
            raise ValueError(f"overlap between {a} and {b} is not smaller than both nodes")
        if ov:
            fa_, fb = ids[a] * 2 + (0 if ap else 1), ids[b] * 2 + (0 if bp else 1)
            breaks.setdefault(fb, set()).add(ov)
            breaks.setdefault(fa_ ^ 1, set()).add(ov)
    pieces = []     # (bignode, offset, sequence)
    lookup = []     # (bignode, [piece indices])
    names = []
    size_of = {}
    for name in order:
        s = seqs[name]
        nid = ids[name]
        for strand, text in ((0, s), (1, s.encode().translate(_COMPLEMENT)[::-1].decode())):
            big = nid * 2 + strand
            idx = []
            bp_ = sorted(breaks.get(big, set()) | {0, len(text)})
            for lo, hi in zip(bp_, bp_[1:]):
                for o in range(lo, hi, SPLIT_NODE_SIZE):
                    idx.append(len(pieces))
                    pieces.append((big, o, text[o:min(o + SPLIT_NODE_SIZE, hi)]))
            lookup.append((big, idx))
            names.append("" if numeric else name)
            size_of[big] = len(text)
    n = len(pieces)
    in_lists = [[] for _ in range(n)]
    out_lists = [[] for _ in range(n)]
    piece_at = {(big, pieces[i][1]): i for big, idx in lookup for i in idx}
    last_piece = {big: idx[-1] for big, idx in lookup}
    for big, idx in lookup:
        for a, b in zip(idx, idx[1:]):
            out_lists[a].append(b)
            in_lists[b].append(a)

    def add_edge(frm, to, ov):
        a, b = last_piece[frm], piece_at[(to, ov)]
        if a not in in_lists[b]:
            in_lists[b].append(a)
        if b not in out_lists[a]:
            out_lists[a].append(b)
    for a, ap, b, bp, ov in links:
        fa_, fb = ids[a] * 2 + (0 if ap else 1), ids[b] * 2 + (0 if bp else 1)
        add_edge(fa_, fb, ov)
        add_edge(fb ^ 1, fa_ ^ 1, ov)
    # ambiguous pieces go to the end in reverse order (RenumberAmbiguousToEnd, AlignmentGraph.cpp:898-985)
    amb = [any(c not in "ACGTUacgtu" for c in p[2]) for p in pieces]
    renum = np.zeros(n, dtype=np.int64)
    na = 0
    nn = 0
    for i in range(n):
        if amb[i]:
            renum[i] = n - 1 - na
            na += 1
        else:
            renum[i] = nn
            nn += 1
    perm = np.empty(n, dtype=np.int64)
    perm[renum] = np.arange(n)
    pieces = [pieces[perm[i]] for i in range(n)]
    in_lists = [[int(renum[x]) for x in in_lists[perm[i]]] for i in range(n)]
    out_lists = [[int(renum[x]) for x in out_lists[perm[i]]] for i in range(n)]
    lookup = [(big, [int(renum[x]) for x in idx]) for big, idx in lookup]
    node_length = np.array([len(p[2]) for p in pieces], dtype=np.uint32)
    node_ids = np.array([p[0] for p in pieces], dtype=np.int32)
    node_offset = np.array([p[1] for p in pieces], dtype=np.uint32)
    reverse = (node_ids % 2 == 1).astype(np.uint8)
    seq2 = np.zeros((nn, 2), dtype=np.uint64)
    for i in range(nn):
        codes = _CODE[np.frombuffer(pieces[i][2].encode(), dtype=np.uint8)].astype(np.uint64)
        for c in range(2):
            part = codes[c * 32:(c + 1) * 32]
            if len(part):
                seq2[i, c] = np.bitwise_or.reduce(part << (2 * np.arange(len(part), dtype=np.uint64)))
    seqa = np.zeros((na, 4), dtype=np.uint64)
    for k in range(na):
        text = pieces[nn + k][2].upper()
        for p_, ch in enumerate(text):
            m = _IUPAC[ch]
            for c in range(4):
                if m >> c & 1:
                    seqa[k, c] |= np.uint64(1 << p_)
    in_off, in_nb = _csr(in_lists)
    out_off, out_nb = _csr(out_lists)
    lin = _find_linearizable(in_lists)
    comp = _component_order(out_lists)
    l_off, l_nodes = _csr([idx for _, idx in lookup])
    chain, chain_pos = _find_chains(n, in_lists, out_lists, comp.tolist(), [idx for _, idx in lookup], node_length)
    return Graph(n, nn, node_length, node_ids, node_offset, reverse, lin, comp,
                 chain, chain_pos,
                 seq2.reshape(-1), seqa.reshape(-1), in_off, in_nb, out_off, out_nb,
                 np.array([b for b, _ in lookup], dtype=np.int32),
                 np.array([size_of[b] for b, _ in lookup], dtype=np.uint32), l_off, l_nodes,
                 names, int(node_length.sum()))
