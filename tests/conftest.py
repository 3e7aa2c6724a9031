import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(autouse=True)
def _fixture_fpmode(monkeypatch):
    """The golden fixtures were made by the reference built on x86-64, whose
    float64 sum keeps the multiply and the add apart; library and oracle
    defaults ("auto": the reference as built on the current host, fused on
    aarch64) are pinned to that mode in every test.  Tests of the host
    default remove the variable themselves."""
    monkeypatch.setenv("CNN_FPMODE", "separate")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


FIT_CASES = [
    "quickstart.npz", "blobs2d_5k.npz", "moons_1500.npz", "varied_1500.npz",
    "varied_nosort.npz", "varied_maxclusters.npz", "edge_grid_boundary.npz",
    "edge_duplicates.npz", "edge_1d.npz", "edge_3d.npz", "edge_single.npz",
    "edge_allnoise.npz", "edge_c0.npz", "highdim_16.npz", "highdim_64.npz",
]


def fit_kwargs(g):
    kw = {}
    if int(g["member_cutoff"]) >= 0:
        kw["member_cutoff"] = int(g["member_cutoff"])
    if int(g["max_clusters"]) >= 0:
        kw["max_clusters"] = int(g["max_clusters"])
    if int(g["cnn_offset"]) != 0:
        kw["cnn_offset"] = int(g["cnn_offset"])
    if not bool(g["sort_by_size"]):
        kw["sort_by_size"] = False
    return kw


@pytest.fixture(scope="session")
def golden():
    return load_golden


def golden_tree(g):
    """Bundles of a stored hierarchy: {path tuple: (labels, root_indices, parent_indices)}."""
    out = {}
    for k, path in enumerate(g["paths"].tolist()):
        key = tuple(int(p) for p in path.split(".")) if path else ()
        lab = g["labels"][g["labels_off"][k]:g["labels_off"][k + 1]]
        root = g["root"][g["root_off"][k]:g["root_off"][k + 1]]
        parent = g["parent"][g["parent_off"][k]:g["parent_off"][k + 1]]
        out[key] = (lab, root, parent)
    return out


def bundle_tree(bundle):
    """The same mapping for a Bundle of this package (labels empty when None)."""
    out = {}
    stack = [((), bundle)]
    while stack:
        path, b = stack.pop()
        lab = np.zeros(0, dtype=np.int64) if b._labels is None else np.asarray(b._labels._host(), dtype=np.int64)
        root = np.zeros(0, dtype=np.int64) if b.root_indices is None else np.asarray(b.root_indices, dtype=np.int64)
        parent = (np.zeros(0, dtype=np.int64) if b.parent_indices is None
                  else np.asarray(b.parent_indices, dtype=np.int64))
        out[path] = (lab, root, parent)
        for label, child in b.children.items():
            stack.append((path + (int(label),), child))
    return out


def predict_cases(g):
    """(points, labels, other, radius_cutoff, cnn_cutoff, clusters or None, expected) per stored case."""
    cases = []
    for k in range(int(g["n_cases"])):
        r, c = g[f"params_{k}"]
        cl = g[f"clusters_{k}"]
        cases.append((g["points"], g[f"labels_{k}"], g["other"], float(r), int(c),
                      cl.tolist() if cl.size else None, g[f"predicted_{k}"]))
    return cases


def pairwise_distances(x):
    """Square Euclidean distances, the expression tests/golden/make_golden.py used."""
    x = np.asarray(x, dtype=np.float64)
    return np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
