"""GPU: HierarchicalFitterMSTPrimGPU (cnn_mst_prim) against the reference's
tree and the oracle's Prim restatement."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import cnn_oracle as o
from test_mst_cpu import bundle_mst, golden_mst

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cnn():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import commonnnclustering_gb300 as cnn
    return cnn


@pytest.mark.parametrize("k", [0, 1])
def test_mst_hierarchy_matches_reference(cnn, k):
    g = load_golden("mst_prim.npz")
    r, mc = g[f"params_{k}"]
    cl = cnn.Clustering(g[f"points_{k}"], hierarchical_fitter="mst")
    cl.fit_hierarchical(radius_cutoff=float(r), member_cutoff=int(mc), v=False)
    assert bundle_mst(cl._bundle) == golden_mst(g, k)


@pytest.mark.parametrize("d,r", [(2, 0.12), (3, 0.25), (5, 0.55)])
def test_mst_edges_against_oracle(cnn, d, r):
    rng = np.random.default_rng(30 + d)
    centres = rng.uniform(-2, 2, size=(5, d))
    x = np.vstack([c + rng.normal(0, 0.3, size=(300, d)) for c in centres] + [rng.uniform(-3, 3, size=(80, d))])
    ctx = cnn.Context(0)
    ctx.set_points(x)
    a, b, w = ctx.mst_prim(r * r)
    want = o.mst_prim_edges(x, r * r)
    assert list(zip(a.tolist(), b.tolist(), w.tolist())) == [(int(p), int(q), int(v)) for p, q, v in want]
    ctx.close()
