import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


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
