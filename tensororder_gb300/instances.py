"""Seeded synthetic CNF instances in DIMACS text (cachet weight lines).

* cubic vertex cover: one variable per vertex of a seeded random 3-regular
  graph, one clause ``(x_u or x_v)`` per edge;
* random 3-CNF: ``floor(ratio * v)`` clauses of 3 distinct variables with
  random polarity.

Weights use the cachet format parsed by ``Formula.parse_DIMACS``
(``util/boolean_formula.py:235-239``): ``w v p`` gives ``w(x)=p`` and
``w(not x)=1-p``.
"""
from __future__ import annotations

import random


def random_regular_graph(d, n, seed):
    """Edges of a seeded random ``d``-regular simple graph (networkx when
    available, which is what the frozen plans were generated with)."""
    import networkx as nx

    g = nx.random_regular_graph(d, n, seed=seed)
    return sorted((min(u, v), max(u, v)) for u, v in g.edges())


def cubic_vertex_cover_cnf(n, seed, weighted=False, lo=0.3, hi=0.7):
    edges = random_regular_graph(3, n, seed)
    rng = random.Random(seed)
    lines = ["p cnf %d %d" % (n, len(edges))]
    if weighted:
        for v in range(1, n + 1):
            lines.append("w %d %r" % (v, rng.uniform(lo, hi)))
    for u, v in edges:
        lines.append("%d %d 0" % (u + 1, v + 1))
    return "\n".join(lines) + "\n"


def random_3cnf(v, ratio, seed, weighted=True, lo=0.2, hi=0.8):
    rng = random.Random(seed)
    m = int(ratio * v)
    lines = ["p cnf %d %d" % (v, m)]
    if weighted:
        for x in range(1, v + 1):
            lines.append("w %d %r" % (x, rng.uniform(lo, hi)))
    for _ in range(m):
        vs = rng.sample(range(1, v + 1), 3)
        lines.append(" ".join(str(x if rng.random() < 0.5 else -x) for x in vs) + " 0")
    return "\n".join(lines) + "\n"


def parse_cnf(text):
    """(num_vars, clauses, {var: (w_neg, w_pos)}) from DIMACS text with cachet
    weights; unweighted variables get (1, 1)."""
    nv = 0
    clauses = []
    weights = {}
    for line in text.splitlines():
        line = line.strip()
        if not line or line[0] == "c":
            continue
        if line[0] == "p":
            nv = int(line.split()[2])
        elif line[0] == "w":
            _, v, p = line.split()[:3]
            p = float(p)
            weights[int(v)] = (1.0, 1.0) if p == -1 else (1.0 - p, p)
        else:
            lits = [int(x) for x in line.split() if int(x) != 0]
            if lits:
                clauses.append(lits)
    return nv, clauses, weights
