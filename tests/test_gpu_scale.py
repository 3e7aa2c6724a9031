"""Parity at the benchmark sizes.

* 200,000 x 3 (cell grid): the whole CSR equals the oracle's and the
  labels equal the oracle's BFS + sort_by_size.
* 500,000 x 64 (tensor cores): the oracle cannot build 2.5e11 pairs in a
  test, so 64 sampled rows are compared against brute-force float64 rows,
  the CSR is checked for size-independent properties (rows ascending,
  symmetric, self included), and the labels equal the oracle's BFS run on
  that checked CSR.
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
    n = x.shape[0]
    deg = np.diff(off)
    assert deg.min() >= 1
    rows = np.repeat(np.arange(n, dtype=np.int64), deg)
    # ascending rows, self included
    assert np.all((np.diff(idx.astype(np.int64)) > 0) | (np.diff(rows) != 0))
    key = rows * n + idx
    assert np.all(np.isin(np.arange(n, dtype=np.int64) * n + np.arange(n), key))
    # symmetric
    assert np.array_equal(np.sort(key), np.sort(idx.astype(np.int64) * n + rows))
    # sampled rows against brute-force float64 rows
    rng = np.random.default_rng(1)
    for i in rng.choice(n, 64, replace=False):
        want = oracle.neighbour_row(x, int(i), r * r)
        assert np.array_equal(idx[off[i]:off[i + 1]], want), i
    # labels: the oracle's BFS on the checked CSR
    want, _ = oracle.clustering_fit(x, r, 8, neighbours=(off, idx))
    assert np.array_equal(labels, want)
