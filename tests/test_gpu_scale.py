"""Parity at the benchmark sizes, against the oracle on the whole workload.

* 200,000 x 3 (cell grid): the whole CSR equals the oracle's and the
  labels equal the oracle's BFS + sort_by_size.
* 500,000 x 64 (tensor cores): the whole CSR equals the oracle's exact
  brute force (the pivot-pruned scan, which evaluates the reference's
  predicate on every pair it cannot rule out by the triangle inequality),
  and the labels equal the oracle's BFS on the oracle's own CSR.
* 1,000,000 x 3 float32-stored, the 8 x 8 batched sweep: the 8 fits at
  cnn_cutoff 10 and the 8 fits at the largest radius equal the oracle's
  fits (grid neighbourhoods + BFS + sort_by_size) on all 1,000,000 points.
"""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def cnn():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import commonnnclustering_gb300 as cnn
    return cnn


@pytest.fixture(scope="module")
def oracle():
    from oracle import cnn_oracle
    return cnn_oracle


def fit_with_csr(cnn, x, r, c, member_cutoff):
    ctx = cnn.Context(0)
    ctx.set_points(x)
    ctx.build_neighbours(r * r)
    off, idx = ctx.get_neighbours(x.shape[0])
    n = x.shape[0]
    labels = np.zeros(n, dtype=np.int64)
    consider = np.ones(n, dtype=np.uint8)
    ctx.fit(c + 2, c + 1, 1, consider, labels)
    ctx.sort_by_size(labels, 2 if member_cutoff is None else member_cutoff, None)
    st = ctx.stats()
    ctx.close()
    return off, idx, labels, st


def test_md3d_200k_full_parity(cnn, oracle):
    from commonnnclustering_gb300 import workloads
    x = workloads.md3d()
    off, idx, labels, st = fit_with_csr(cnn, x, 0.1, 10, 50)
    assert st["search_kind"] == 1
    want_off, want_idx = oracle.neighbourhoods(x, 0.1 ** 2)
    assert np.array_equal(off, want_off) and np.array_equal(idx, want_idx)
    want, _ = oracle.clustering_fit(x, 0.1, 10, member_cutoff=50, neighbours=(want_off, want_idx))
    assert np.array_equal(labels, want)


def test_features_500k_d64_parity(cnn, oracle):
    from commonnnclustering_gb300 import workloads
    x = workloads.features()
    r = 2.9
    off, idx, labels, st = fit_with_csr(cnn, x, r, 8, None)
    assert st["search_kind"] == 3, st
    want_off, want_idx = oracle.neighbourhoods(x, r * r, grid="pivot")
    assert np.array_equal(off, want_off)
    assert np.array_equal(idx, want_idx)
    want, _ = oracle.clustering_fit(x, r, 8, neighbours=(want_off, want_idx))
    assert np.array_equal(labels, want)


def test_nested3d_1m_sweep_against_oracle(cnn, oracle):
    from commonnnclustering_gb300 import workloads
    x = workloads.nested3d()  # float32-stored, widened exactly
    x64 = x.astype(np.float64)
    radii = [float(r) for r in np.linspace(0.03, 0.15, 8)]
    cuts = [2, 5, 10, 20, 40, 80, 120, 160]
    got = cnn.sweep(x, radii, cuts, member_cutoff=2)
    assert got.shape == (8, 8, x.shape[0])
    for k, r in enumerate(radii):
        csr = oracle.neighbourhoods(x64, r * r)
        for j, c in enumerate(cuts):
            if c != 10 and k != len(radii) - 1:
                continue
            want, _ = oracle.clustering_fit(x64, r, c, member_cutoff=2, neighbours=csr)
            assert np.array_equal(got[k, j], want), (r, c)
        del csr
