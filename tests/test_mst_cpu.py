"""HierarchicalFitterMSTPrimGPU's hierarchy bookkeeping against the tree the
reference built (tests/golden/mst_prim.npz).  The spanning-forest edges come
from the oracle's restatement of the reference's Prim loop here (no GPU)."""
from collections import deque

import numpy as np
import pytest

from conftest import load_golden
from oracle import cnn_oracle as o


def golden_mst(g, k):
    out = {}
    for i, path in enumerate(g[f"paths_{k}"].tolist()):
        nodes = g[f"nodes_{k}"][g[f"nodes_off_{k}"][i]:g[f"nodes_off_{k}"][i + 1]]
        edges = g[f"edges_{k}"][g[f"edges_off_{k}"][i]:g[f"edges_off_{k}"][i + 1]]
        out[path] = (nodes.tolist(), [tuple(e) for e in edges.tolist()], float(g[f"lambdas_{k}"][i]))
    return out


def bundle_mst(root):
    out = {}
    q = deque([((), root)])
    while q:
        path, b = q.popleft()
        gr = b._graph
        nodes = sorted(gr.nodes) if gr is not None else []
        edges = sorted((min(u, v), max(u, v), float(d["weight"])) for u, v, d in gr.edges(data=True)) \
            if gr is not None else []
        out[".".join(str(p) for p in path)] = (nodes, edges, float(b._lambda))
        for label in sorted(b.children):
            q.append((path + (label,), b.children[label]))
    return out


@pytest.mark.parametrize("k", [0, 1])
def test_mst_hierarchy_matches_reference(monkeypatch, k):
    import commonnnclustering_gb300 as cnn
    g = load_golden("mst_prim.npz")
    x = g[f"points_{k}"]
    r, mc = g[f"params_{k}"]

    def oracle_edges(self, input_data, radius_cutoff):
        return o.mst_prim_edges(input_data.data, radius_cutoff)

    monkeypatch.setattr(cnn.HierarchicalFitterMSTPrimGPU, "tree_edges", oracle_edges)
    cl = cnn.Clustering(x, hierarchical_fitter="mst")
    cl.fit_hierarchical(radius_cutoff=float(r), member_cutoff=int(mc), v=False)
    assert bundle_mst(cl._bundle) == golden_mst(g, k)


def test_weighted_graph_interface():
    import commonnnclustering_gb300 as cnn
    gr = cnn.WeightedGraph([(3, 1, {"weight": 4.0})])
    gr.add_edges_from([(1, 5, {"weight": 2.0})])
    assert len(gr) == 3 and sorted(gr.nodes) == [1, 3, 5]
    assert sorted(gr.edges(data=True)) == [(1, 3, {"weight": 4.0}), (1, 5, {"weight": 2.0})]
