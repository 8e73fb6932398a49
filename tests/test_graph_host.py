"""Execution graph analysis on the host (no GPU): the reference's hazard-analyzer
and scheduler unit tests (tests/unit/runtime/test_hazard_analyzer.cpp,
test_topological_scheduler.cpp) replayed through the C ABI, plus the
topological order against a plain Kahn restatement on random DAGs."""
import collections
import time

import numpy as np
import pytest

from fluidloom_gb300 import graph as G
from fluidloom_gb300.runtime import FluidLoomError


def kernel(g, name, reads=(), writes=(), level=-1):
    return g.add(G.KERNEL, name, reads=reads, writes=writes, level=level)


def test_detect_raw():  # test_hazard_analyzer.cpp:21-42
    g = G.Graph()
    a = kernel(g, "NodeA", writes=["density"])
    b = kernel(g, "NodeB", reads=["density"])
    hz = g.analyze()
    assert (a, b, G.RAW, "density") in hz


def test_detect_waw():  # :44-65
    g = G.Graph()
    a = kernel(g, "NodeA", writes=["density"])
    b = kernel(g, "NodeB", writes=["density"])
    assert (a, b, G.WAW, "density") in g.analyze()


def test_detect_war():  # :67-88
    g = G.Graph()
    a = kernel(g, "NodeA", reads=["density"])
    b = kernel(g, "NodeB", writes=["density"])
    assert (a, b, G.WAR, "density") in g.analyze()


def test_detect_level_barrier():  # :90-111
    g = G.Graph()
    kernel(g, "NodeA", level=0)
    kernel(g, "NodeB", level=1)
    assert any(h[2] == G.LEVEL_BARRIER for h in g.analyze())


def test_no_false_positives():  # :113-132
    g = G.Graph()
    kernel(g, "NodeA", reads=["density"], writes=["velocity"])
    kernel(g, "NodeB", reads=["pressure"], writes=["density"])
    hz = g.analyze()
    assert len(hz) == 1 and hz[0][2] == G.WAR


def simple_dag():
    g = G.Graph()
    a, b, c = kernel(g, "A"), kernel(g, "B"), kernel(g, "C")
    g.add_edge(a, b)
    g.add_edge(b, c)
    return g, (a, b, c)


def test_simple_dag_order():  # test_topological_scheduler.cpp:53-74
    g, (a, b, c) = simple_dag()
    g.build()
    order = g.order()
    assert len(order) == 3 and order.index(a) < order.index(b) < order.index(c)
    assert g.num_edges() == 2


def complex_dag(n):
    g = G.Graph()
    ids = [kernel(g, "Node%d" % i) for i in range(n)]
    for i in range(2, n):  # each node depends on the previous two (:33-51)
        g.add_edge(ids[i - 1], ids[i])
        g.add_edge(ids[i - 2], ids[i])
    return g, ids


def test_complex_dag_and_build_time():  # :76-101
    g, ids = complex_dag(100)
    t0 = time.perf_counter()
    g.build()
    ms = (time.perf_counter() - t0) * 1e3
    order = g.order()
    assert sorted(order) == ids
    pos = {v: k for k, v in enumerate(order)}
    for i in range(2, 100):
        assert pos[ids[i - 2]] < pos[ids[i]] and pos[ids[i - 1]] < pos[ids[i]]
    assert ms < 1.0


def test_cycle_detection():  # :103-126
    g, (a, b, c) = simple_dag()
    g.add_edge(c, a)
    with pytest.raises(FluidLoomError, match="cycles"):
        g.build()
    with pytest.raises(FluidLoomError):
        g.order()  # "Graph not yet validated"


def kahn(n, edges):
    """Kahn's algorithm with a FIFO ready queue (DependencyGraphBuilder.cpp:62-99)."""
    succ = collections.defaultdict(list)
    indeg = [0] * n
    for a, b in edges:
        succ[a].append(b)
        indeg[b] += 1
    q = collections.deque(i for i in range(n) if indeg[i] == 0)
    out = []
    while q:
        i = q.popleft()
        out.append(i)
        for s in succ[i]:
            indeg[s] -= 1
            if indeg[s] == 0:
                q.append(s)
    return out


def hazards_ref(nodes):
    """The analyzer's pair scan in its order: RAW, WAW, WAR, level barriers."""
    out = []
    for kind, (fa, fb) in ((G.RAW, ("w", "r")), (G.WAW, ("w", "w")), (G.WAR, ("r", "w"))):
        for i in range(len(nodes)):
            for j in range(i + 1, len(nodes)):
                for f in nodes[i][fa]:
                    if f in nodes[j][fb]:
                        out.append((i, j, kind, f))
    for i in range(len(nodes)):
        if nodes[i]["l"] < 0:
            continue
        for j in range(i + 1, len(nodes)):
            if nodes[j]["l"] >= 0 and nodes[j]["l"] != nodes[i]["l"]:
                out.append((i, j, G.LEVEL_BARRIER, ""))
    return out


@pytest.mark.parametrize("seed", range(5))
def test_random_graphs_match_restatement(seed):
    rng = np.random.default_rng(seed)
    fields = ["f%d" % k for k in range(6)]
    n = int(rng.integers(5, 40))
    nodes = []
    g = G.Graph()
    for i in range(n):
        r = [f for f in fields if rng.random() < 0.2]
        w = [f for f in fields if rng.random() < 0.15]
        lv = int(rng.integers(-1, 3))
        nodes.append({"r": r, "w": w, "l": lv})
        kernel(g, "n%d" % i, reads=r, writes=w, level=lv)
    extra = [(int(a), int(b)) for a, b in rng.integers(0, n, (n // 2, 2)) if a < b]
    for a, b in extra:
        g.add_edge(a, b)
    hz = g.analyze()
    assert hz == hazards_ref(nodes)
    g.build()
    edges = extra + [(h[0], h[1]) for h in hz]
    assert g.order() == kahn(n, edges)
    assert g.num_edges() == len(edges)
    assert g.dot().startswith("digraph DependencyGraph {")
