"""Strong-coupling diagram topologies (chord diagrams) and their parities.

Restates `src/diagrammatics.jl:46-337`: a topology of order n pairs the vertices
1..2n into n arcs (a_1 < b_1 for every arc as generated), its parity is the sign of the
flattened permutation, and `get_topologies_at_order(n, k)` keeps the doubly
k-connected ones (`:231-235`), optionally flipping the parity by (-1)^k for an external
arc (`:332-334`).  Vertex numbering and generation order are the reference's, so the
topology lists (and therefore summation order) agree.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Tuple

Pair = Tuple[int, int]


@dataclass(frozen=True)
class Topology:
    order: int
    pairs: Tuple[Pair, ...]
    parity: int


def _generate(partial: List[Pair], parity: int, unpaired: List[int], out: List[Topology]):
    # src/diagrammatics.jl:288-299: pair the first unpaired vertex with the i-th one
    # (1-based i = 2..len); each step flips the parity by (-1)^i.
    if not unpaired:
        out.append(Topology(len(partial), tuple(partial), parity))
        return
    for i in range(2, len(unpaired) + 1):
        p = (unpaired[0], unpaired[i - 1])
        rest = [unpaired[k] for k in range(len(unpaired)) if k not in (0, i - 1)]
        _generate(partial + [p], parity * (-1) ** i, rest, out)


def generate_topologies(n: int) -> List[Topology]:
    out: List[Topology] = []
    _generate([], 1, list(range(1, 2 * n + 1)), out)
    return out


def _sortpair(p: Pair) -> Pair:
    return (p[1], p[0]) if p[0] > p[1] else p


def iscrossing(p1: Pair, p2: Pair) -> bool:
    a1, b1 = _sortpair(p1)
    a2, b2 = _sortpair(p2)
    return (a1 < a2 < b1 < b2) or (a2 < a1 < b2 < b1)


def is_doubly_k_connected_pair(p: Pair, k: int) -> bool:
    return (p[0] <= k < p[1]) or (p[1] <= k < p[0])


def _traverse_crossing_graph(connected: List[Pair], disconnected: List[Pair]) -> None:
    stack = list(connected)
    connected.clear()
    while stack:
        pc = stack.pop()
        connected.append(pc)
        for i in range(len(disconnected) - 1, -1, -1):
            if iscrossing(pc, disconnected[i]):
                stack.append(disconnected.pop(i))


def is_doubly_k_connected(top: Topology, k: int) -> bool:
    con = [p for p in top.pairs if is_doubly_k_connected_pair(p, k)]
    dis = [p for p in top.pairs if not is_doubly_k_connected_pair(p, k)]
    _traverse_crossing_graph(con, dis)
    return not dis


def is_k_connected(top: Topology, k: int) -> bool:
    con = [p for p in top.pairs if p[0] <= k or p[1] <= k]
    dis = [p for p in top.pairs if not (p[0] <= k or p[1] <= k)]
    _traverse_crossing_graph(con, dis)
    return not dis


def count_doubly_k_connected(pairs, k: int) -> int:
    return sum(1 for p in pairs if is_doubly_k_connected_pair(p, k))


def get_topologies_at_order(order: int, k: Optional[int] = None,
                            with_external_arc: bool = False) -> List[Topology]:
    tops = generate_topologies(order)
    if k is None:
        return tops
    tops = [t for t in tops if is_doubly_k_connected(t, k)]
    if with_external_arc:
        tops = [Topology(t.order, t.pairs, (-1) ** k * t.parity) for t in tops]
    return tops


def levicivita(perm) -> int:
    perm = list(perm)
    sign = 1
    seen = [False] * len(perm)
    for i in range(len(perm)):
        if seen[i]:
            continue
        j = i
        length = 0
        while not seen[j]:
            seen[j] = True
            j = perm[j] - 1
            length += 1
        if length % 2 == 0:
            sign = -sign
    return sign


def isvalid(top: Topology) -> bool:
    perm = [v for p in top.pairs for v in p]
    return top.parity == levicivita(perm) and sorted(perm) == list(range(1, 2 * top.order + 1))
