"""The cell-grid neighbour graph in mask form (one bit per stencil candidate,
the bitset intersection) against the same graph as sorted lists (the merge
intersection): identical neighbour lists, labels, consider flags and check
counts, over dimensions, cutoffs and edge cases; the tuner that picks
between them; the MST weights taken from the masks.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def abi():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from commonnnclustering_gb300 import _abi
    return _abi


def context(abi, monkeypatch, form):
    ctx = abi.Context(0)
    ctx.set_intersection(abi.INTERSECT_MERGE if form == "lists" else abi.INTERSECT_BITSET)
    return ctx


def fit(ctx, x, r2, sc, nm, consider=None, labels=None):
    n = x.shape[0]
    lab = np.zeros(n, dtype=np.int64) if labels is None else labels.copy()
    con = np.ones(n, dtype=np.uint8) if consider is None else consider.copy()
    ctx.set_points(x)
    ctx.build_neighbours(r2)
    ctx.fit(sc, nm, 7, con, lab)
    return lab, con, ctx.stats()


CASES = []
rng = np.random.default_rng(77)
CASES.append(("blobs2d", None, 0.3 ** 2))
CASES.append(("md3d", None, 0.1 ** 2))
CASES.append(("line1d", np.sort(rng.uniform(0, 50, size=(6000, 1)), axis=0), 0.05 ** 2))
CASES.append(("dups3d", np.repeat(rng.normal(size=(1500, 3)), 3, axis=0), 0.3 ** 2))
CASES.append(("lattice2d", np.stack(np.meshgrid(np.arange(60.0), np.arange(60.0)), -1).reshape(-1, 2) * 0.5, 0.25))
CASES.append(("wide3d", rng.uniform(-40, 40, size=(20000, 3)), 2.5 ** 2))


def points(name, x):
    from commonnnclustering_gb300 import workloads
    if name == "blobs2d":
        return workloads.blobs2d()
    if name == "md3d":
        return workloads.md3d(n=40000, seed=11, centre_spread=2.0)
    return np.ascontiguousarray(x)


@pytest.mark.parametrize("name,x,r2", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("c,m", [(0, 0), (1, 1), (5, 3), (20, 8), (-1, 2)])
def test_masks_equal_lists(abi, monkeypatch, name, x, r2, c, m):
    x = points(name, x)
    a = context(abi, monkeypatch, "masks")
    b = context(abi, monkeypatch, "lists")
    sc, nm = (c + 2 if c >= 0 else -5), m + 1
    la, ca, sa = fit(a, x, r2, sc, nm)
    lb, cb, sb = fit(b, x, r2, sc, nm)
    assert np.array_equal(la, lb) and np.array_equal(ca, cb)
    for k in ("n_nonzero", "n_nodes", "n_candidates", "n_exact"):
        assert sa[k] == sb[k], k
    oa, ia = a.get_neighbours(x.shape[0])
    ob, ib = b.get_neighbours(x.shape[0])
    assert np.array_equal(oa, ob) and np.array_equal(ia, ib)
    # a fit after the lists were made from the masks is still the mask fit
    la2, _, _ = fit(a, x, r2, sc, nm)
    assert np.array_equal(la2, la)
    a.close()
    b.close()


def test_masks_with_consider_and_non_finite_points(abi, monkeypatch):
    from commonnnclustering_gb300 import workloads
    x = workloads.md3d(n=30000, seed=13, centre_spread=2.0)
    x[::97, 1] = np.nan
    x[5::131, 0] = np.inf
    r = np.random.default_rng(1)
    consider = (r.random(x.shape[0]) < 0.8).astype(np.uint8)
    labels = np.where(consider == 0, 3, 0).astype(np.int64)
    a = context(abi, monkeypatch, "masks")
    b = context(abi, monkeypatch, "lists")
    la, ca, _ = fit(a, x, 0.1 ** 2, 12, 9, consider, labels)
    lb, cb, _ = fit(b, x, 0.1 ** 2, 12, 9, consider, labels)
    assert np.array_equal(la, lb) and np.array_equal(ca, cb)
    from oracle import cnn_oracle
    want = cnn_oracle.neighbourhoods(x, 0.1 ** 2)
    off, idx = a.get_neighbours(x.shape[0])
    assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])
    a.close()
    b.close()


def test_tuner_times_both_forms_once_per_profile(abi):
    """Under INTERSECT_AUTO the first fit of a profile runs both strategies
    (tuned = 1, labels as the merge gives them); later graphs of the same
    profile are built in the chosen form only and fitted with it."""
    from commonnnclustering_gb300 import workloads
    x = workloads.md3d(n=37000, seed=17, centre_spread=2.0)
    ref = abi.Context(0)
    ref.set_intersection(abi.INTERSECT_MERGE)
    want, wcon, _ = fit(ref, x, 0.1 ** 2, 12, 11)
    ctx = abi.Context(0)
    ctx.set_intersection(abi.INTERSECT_AUTO)
    seen = []
    for _ in range(3):
        lab, con, st = fit(ctx, x, 0.1 ** 2, 12, 11)
        assert np.array_equal(lab, want) and np.array_equal(con, wcon)
        assert st["intersection"] in (abi.INTERSECT_MERGE, abi.INTERSECT_BITSET)
        seen.append((st["tuned"], st["intersection"], st["tune_ms_merge"], st["tune_ms_bitset"]))
    tuned = [t for t, *_ in seen]
    assert tuned.count(1) <= 1 and tuned[1:] == [0, 0]  # the profile may be known from an earlier test
    assert seen[1][1] == seen[2][1]
    if tuned[0] == 1:
        merge, bitset = seen[0][2], seen[0][3]
        assert merge > 0 and bitset > 0
        assert seen[1][1] == (abi.INTERSECT_BITSET if bitset < merge else abi.INTERSECT_MERGE)
    ctx.close()
    ref.close()


def test_mst_weights_from_masks_equal_the_merge(abi):
    from commonnnclustering_gb300 import workloads
    from oracle import cnn_oracle
    x = workloads.blobs2d(n=1000, seed=9)
    out = {}
    for strat in (abi.INTERSECT_MERGE, abi.INTERSECT_BITSET):
        ctx = abi.Context(0)
        ctx.set_intersection(strat)
        ctx.set_points(x)
        out[strat] = ctx.mst_prim(0.3 ** 2)
        assert ctx.stats()["intersection"] == strat
        ctx.close()
    for a, b in zip(out[abi.INTERSECT_MERGE], out[abi.INTERSECT_BITSET]):
        assert np.array_equal(a, b)
    want = np.asarray(cnn_oracle.mst_prim_edges(x, 0.3 ** 2), dtype=np.int64).reshape(-1, 3)
    got = np.stack(out[abi.INTERSECT_BITSET], axis=1)
    assert np.array_equal(got, want)
