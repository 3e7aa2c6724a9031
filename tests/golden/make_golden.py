"""Generate the golden fixtures in this folder by running the REFERENCE.

The reference (cnnclustering 0.5.0) is a Cython package.  It is installed
from its source tree into ``baseline/_ref`` once, without network:

    cp -r <reference checkout> /tmp/refsrc
    python -m pip install --no-index --no-build-isolation --no-deps \
        --find-links /opt/wheelhouse --target baseline/_ref /tmp/refsrc

and then this script imports it from there (x86-64 build, GCC, baseline
ISA: the distance sum is computed with a separate multiply and add).
Run from the repository root:

    python tests/golden/make_golden.py

Every fixture stores the inputs next to the reference's outputs, so the
tests need neither the reference nor scikit-learn at run time.
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "baseline", "_ref"))
sys.path.insert(0, ROOT)

from cnnclustering import cluster, _types, _fit  # noqa: E402
from cnnclustering._types import Labels, ClusterParameters  # noqa: E402

from commonnnclustering_gb300 import workloads  # noqa: E402


def csr_digest(offsets: np.ndarray, indices: np.ndarray) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(offsets, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(indices, dtype=np.int32).tobytes())
    return h.hexdigest()


def reference_neighbourhoods(x: np.ndarray, r: float, metric: str = "euclidean_r"):
    """Rows of the reference's own brute-force getter, index order."""
    metric_type = {"euclidean_r": _types.MetricExtEuclideanReduced,
                   "euclidean": _types.MetricExtEuclidean}[metric]
    m = metric_type()
    getter = _types.NeighboursGetterExtBruteForce(_types.DistanceGetterExtMetric(m))
    data = _types.InputDataExtComponentsMemoryview(np.ascontiguousarray(x, dtype=np.float64))
    radius = r * r if metric == "euclidean_r" else r
    params = ClusterParameters(radius)
    nb = _types.NeighboursExtVector(64)
    rows = []
    for i in range(x.shape[0]):
        getter.get(i, data, nb, params)
        rows.append(np.array([nb.get_member(k) for k in range(nb.n_points)], dtype=np.int32))
    offsets = np.zeros(x.shape[0] + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([len(a) for a in rows])
    indices = np.concatenate(rows) if rows else np.zeros(0, dtype=np.int32)
    return offsets, indices


def ref_fit(x, r, c, recipe="coordinates", **fit_kwargs):
    cl = cluster.Clustering(np.ascontiguousarray(x, dtype=np.float64), recipe=recipe)
    t = time.time()
    cl.fit(r, c, v=False, **fit_kwargs)
    return np.array(cl.labels, dtype=np.int64), time.time() - t


def ref_fit_metric(x, r, c, metric_type, **fit_kwargs):
    recipe = {
        "input_data": _types.InputDataExtComponentsMemoryview,
        "fitter": _fit.FitterExtBFS,
        "fitter.ngetter": _types.NeighboursGetterExtBruteForce,
        "fitter.na": _types.NeighboursExtVectorCPPUnorderedSet,
        "fitter.checker": _types.SimilarityCheckerExtSwitchContains,
        "fitter.queue": _types.QueueExtFIFOQueue,
        "fitter.ngetter.dgetter": _types.DistanceGetterExtMetric,
        "fitter.ngetter.dgetter.metric": metric_type,
    }
    cl = cluster.Clustering(np.ascontiguousarray(x, dtype=np.float64), recipe=recipe)
    cl.fit(r, c, v=False, **fit_kwargs)
    return np.array(cl.labels, dtype=np.int64)


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, {k: getattr(v, "shape", v) for k, v in arrays.items()})


def fit_case(name, x, r, c, store_csr=True, fit_kwargs=None):
    fit_kwargs = dict(fit_kwargs or {})
    labels, t = ref_fit(x, r, c, **fit_kwargs)
    offsets, indices = reference_neighbourhoods(x, r)
    arrays = dict(points=np.asarray(x, dtype=np.float64), labels=labels,
                  radius_cutoff=np.float64(r), cnn_cutoff=np.int64(c),
                  member_cutoff=np.int64(fit_kwargs.get("member_cutoff", -1)),
                  max_clusters=np.int64(fit_kwargs.get("max_clusters", -1) or -1),
                  cnn_offset=np.int64(fit_kwargs.get("cnn_offset", 0) or 0),
                  sort_by_size=np.bool_(fit_kwargs.get("sort_by_size", True)),
                  degrees=np.diff(offsets).astype(np.int32),
                  csr_sha256=np.array(csr_digest(offsets, indices)),
                  ref_fit_seconds=np.float64(t))
    if store_csr:
        arrays["offsets"] = offsets
        arrays["indices"] = indices
    # the sorted-neighbourhoods recipe on the same lists must agree
    cl = cluster.Clustering([indices[offsets[i]:offsets[i + 1]] for i in range(x.shape[0])],
                            recipe="sorted_neighbourhoods")
    cl.fit(r, c, v=False, **fit_kwargs)
    assert np.array_equal(np.asarray(cl.labels), labels), name
    save(name, **arrays)


def main():
    # 1. README quickstart (README.md:71-93)
    q = np.array([[0, 0], [1, 1], [1, 0], [0, -1], [0.5, -0.5], [2, 1.5], [2.5, -0.5],
                  [4, 2], [4.5, 2.5], [5, -1], [5.5, -0.5], [5.5, -1.5]], dtype=np.float64)
    fit_case("quickstart.npz", q, 1.5, 1)

    # 2. the 5,000-point 2D blobs workload, default recipe (brute force)
    x = workloads.blobs2d()
    fit_case("blobs2d_5k.npz", x, 0.3, 5, store_csr=False, fit_kwargs={"member_cutoff": 10})

    # 3./4. the integration-test toy sets (test/integration/test_procedures.py:126-139)
    from sklearn import datasets
    from sklearn.preprocessing import StandardScaler
    pts, _ = datasets.make_moons(n_samples=1500, random_state=0)
    pts = StandardScaler().fit_transform(pts)
    fit_case("moons_1500.npz", pts, 0.2, 5)
    pts, _ = datasets.make_blobs(n_samples=1500, cluster_std=[1.0, 2.5, 0.5], random_state=170)
    pts = StandardScaler().fit_transform(pts)
    fit_case("varied_1500.npz", pts, 0.25, 20, fit_kwargs={"member_cutoff": 20})

    # 5. fit options: no sorting, max_clusters, cnn_offset
    fit_case("varied_nosort.npz", pts, 0.25, 20, fit_kwargs={"sort_by_size": False})
    fit_case("varied_maxclusters.npz", pts, 0.25, 10,
             fit_kwargs={"member_cutoff": 5, "max_clusters": 2, "cnn_offset": 2})

    # 6. non-reduced Euclidean metric (sqrt then compare with r)
    rng = np.random.default_rng(11)
    xe = np.vstack([rng.normal(0, 0.4, size=(300, 3)), rng.normal(2, 0.3, size=(200, 3)),
                    rng.uniform(-2, 4, size=(100, 3))])
    lab_e = ref_fit_metric(xe, 0.35, 4, _types.MetricExtEuclidean, member_cutoff=5)
    off_e, idx_e = reference_neighbourhoods(xe, 0.35, metric="euclidean")
    save("euclidean_sqrt.npz", points=xe, labels=lab_e, radius_cutoff=np.float64(0.35),
         cnn_cutoff=np.int64(4), member_cutoff=np.int64(5), offsets=off_e, indices=idx_e)

    # 7. frozen labels: fit, freeze, refit the unassigned points
    pts, _ = datasets.make_moons(n_samples=800, noise=0.08, random_state=3)
    pts = StandardScaler().fit_transform(pts)
    cl = cluster.Clustering(pts)
    cl.fit(0.25, 8, v=False, member_cutoff=5)
    first = np.array(cl.labels, dtype=np.int64)
    cl._bundle._labels.meta["frozen"] = True
    consider = (first == 0).astype(np.uint8)
    cl._bundle._labels.consider[:] = consider
    cl.fit(0.35, 3, v=False, member_cutoff=2)
    second = np.array(cl.labels, dtype=np.int64)
    save("frozen_refit.npz", points=pts, first_labels=first, consider=consider,
         second_labels=second, r1=np.float64(0.25), c1=np.int64(8), m1=np.int64(5),
         r2=np.float64(0.35), c2=np.int64(3), m2=np.int64(2))

    # 8. sort_by_size vectors (test/unit/test_types.py:98-117) plus random ones
    base = np.array([1, 1, 2, 2, 0, 1, 3, 3, 3, 1, 5], dtype=np.int64)
    cases = [({"member_cutoff": 1}, base), ({}, base),
             ({"member_cutoff": 2, "max_clusters": 2}, base)]
    rng = np.random.default_rng(5)
    for k in range(6):
        lab = rng.integers(0, 9, size=200).astype(np.int64)
        cases.append(({"member_cutoff": int(k % 4), "max_clusters": (None if k < 3 else 3 + k)}, lab))
    lab = rng.integers(0, 3000, size=5000).astype(np.int64) * 7 - 50
    lab[rng.random(5000) < 0.2] = 0
    cases.append(({"member_cutoff": 2}, lab))
    ins, outs, mcs, mxs = [], [], [], []
    for kw, lab in cases:
        L = Labels(lab.copy())
        L.sort_by_size(**kw)
        ins.append(lab)
        outs.append(np.asarray(L.labels).copy())
        mcs.append(-1 if kw.get("member_cutoff") is None else kw["member_cutoff"])
        mxs.append(-1 if kw.get("max_clusters") is None else kw["max_clusters"])
    save("sort_by_size.npz", n_cases=np.int64(len(cases)),
         member_cutoff=np.array(mcs, dtype=np.int64), max_clusters=np.array(mxs, dtype=np.int64),
         **{f"in_{i}": a for i, a in enumerate(ins)}, **{f"out_{i}": a for i, a in enumerate(outs)})

    # 9. similarity check truth table (test/unit/test_check_similarity.py:38-48)
    #    on sorted members with the screensorted checker, plus random lists
    table = [([], [], 0), ([], [], 1), ([1, 2, 3], [2, 5], 1), ([1, 2, 3], [2, 5, 8, 9], 2),
             ([1, 2, 3, 9, 10], [2, 5, 8, 9, 10], 3), ([1, 2, 3, 9, 10, 18], [2, 5, 8, 9, 10, 11, 18], 3)]
    for k in range(40):
        a = np.unique(rng.integers(0, 200, size=rng.integers(1, 120)))
        b = np.unique(rng.integers(0, 200, size=rng.integers(1, 120)))
        table.append((a.tolist(), b.tolist(), int(rng.integers(0, 40))))
    checker = _types.SimilarityCheckerExtScreensorted()
    res, flat_a, flat_b, la, lb, cs = [], [], [], [], [], []
    for a, b, c in table:
        na_, nb_ = _types.NeighboursExtVector(8), _types.NeighboursExtVector(8)
        for m in a:
            na_.assign(m)
        for m in b:
            nb_.assign(m)
        res.append(bool(checker.check(na_, nb_, ClusterParameters(0.0, similarity_cutoff=c))))
        flat_a += list(a); flat_b += list(b); la.append(len(a)); lb.append(len(b)); cs.append(c)
    save("check_table.npz", a=np.array(flat_a, dtype=np.int32), b=np.array(flat_b, dtype=np.int32),
         len_a=np.array(la, dtype=np.int64), len_b=np.array(lb, dtype=np.int64),
         c=np.array(cs, dtype=np.int64), expected=np.array(res, dtype=np.bool_))

    # 10. edge cases: exact-boundary distances, duplicates, 1-D and 3-D, tiny sets
    g = np.array([[i, j] for i in range(8) for j in range(8)], dtype=np.float64)
    fit_case("edge_grid_boundary.npz", g, 1.0, 2)            # s == r**2 exactly for lattice neighbours
    dup = np.repeat(rng.normal(size=(40, 2)), 3, axis=0)
    fit_case("edge_duplicates.npz", dup, 0.3, 2)
    line = np.sort(rng.uniform(0, 10, size=300))[:, None]
    fit_case("edge_1d.npz", line, 0.15, 3)
    cube = np.vstack([rng.normal(0, 0.2, size=(250, 3)), rng.normal(1.5, 0.25, size=(250, 3))])
    fit_case("edge_3d.npz", cube, 0.2, 6, fit_kwargs={"member_cutoff": 3})
    fit_case("edge_single.npz", np.zeros((1, 2)), 0.5, 0)
    fit_case("edge_allnoise.npz", rng.uniform(0, 100, size=(60, 2)), 0.5, 1)
    fit_case("edge_c0.npz", cube[:200], 0.15, 0, fit_kwargs={"member_cutoff": 1})

    # 11. higher dimensions (the generic / Gram neighbour search paths)
    for d in (16, 64):
        xh = workloads.features(n=600, d=d, seed=7, n_clusters=6)
        dist = np.sqrt(((xh[:50, None, :] - xh[None, :, :]) ** 2).sum(-1))
        r = float(np.quantile(np.sort(dist, axis=1)[:, 25], 0.5))
        fit_case(f"highdim_{d}.npz", xh, r, 5, fit_kwargs={"member_cutoff": 5})

    # 12. HierarchicalFitterRepeat: a step list of fits, the bundle tree it
    # builds (labels and reference indices per bundle) and reel()
    hierarchy_case(rng)

    # 13. PredictorFirstmatch on coordinates (brute-force getters)
    predict_case(rng)

    # 14. the periodic metric and precomputed distances (square and linear)
    metric_input_cases(rng)

    # 15. HierarchicalFitterMSTPrim: the bundle tree of a maximum spanning forest
    mst_case(rng)


def hierarchy_tree(root):
    """Bundles of the tree, breadth first: path, labels, root/parent indices."""
    from collections import deque
    paths, labels, root_idx, parent_idx = [], [], [], []
    q = deque([((), root)])
    while q:
        path, b = q.popleft()
        paths.append(".".join(str(p) for p in path))
        lab = b.labels
        labels.append(np.asarray(lab, dtype=np.int64) if lab is not None else np.zeros(0, dtype=np.int64))
        ri = b.root_indices
        pi = b.parent_indices
        root_idx.append(np.asarray(ri, dtype=np.int64) if ri is not None else np.zeros(0, dtype=np.int64))
        parent_idx.append(np.asarray(pi, dtype=np.int64) if pi is not None else np.zeros(0, dtype=np.int64))
        for label in sorted(b.children):
            q.append((path + (label,), b.children[label]))

    def pack(arrs):
        off = np.zeros(len(arrs) + 1, dtype=np.int64)
        off[1:] = np.cumsum([a.shape[0] for a in arrs])
        return off, (np.concatenate(arrs) if arrs else np.zeros(0, dtype=np.int64))

    lo, lv = pack(labels)
    ro, rv = pack(root_idx)
    po, pv = pack(parent_idx)
    return {"paths": np.array(paths), "labels_off": lo, "labels": lv, "root_off": ro, "root": rv,
            "parent_off": po, "parent": pv}


def hierarchy_case(rng):
    parents = rng.uniform(-6, 6, size=(5, 2))
    kids = (parents[:, None, :] + rng.normal(0, 0.8, size=(5, 3, 2))).reshape(-1, 2)
    x = np.vstack([k + rng.normal(0, 0.18, size=(120, 2)) for k in kids])
    x = x[rng.permutation(x.shape[0])]
    # the repeat fitter passes (radius_cutoff, cnn_cutoff) through unadjusted:
    # the reduced metric compares squared distances with radius_cutoff itself
    radii = np.array([0.5, 0.12, 0.05], dtype=np.float64)
    cuts = np.array([4, 6, 8], dtype=np.int64)
    recipe = {"input_data": "components_mview", "preparation_hook": "points_from_parts",
              "hierarchical_fitter": "repeat", "hierarchical_fitter.fitter": "bfs",
              "hierarchical_fitter.fitter.ngetter": "brute_force", "hierarchical_fitter.fitter.na": "vuset",
              "hierarchical_fitter.fitter.checker": "switch", "hierarchical_fitter.fitter.queue": "fifo",
              "hierarchical_fitter.fitter.ngetter.dgetter": "metric",
              "hierarchical_fitter.fitter.ngetter.dgetter.metric": "euclidean_r"}
    cl = cluster.Clustering(np.ascontiguousarray(x), recipe=recipe)
    cl.fit_hierarchical(radius_cutoff=list(radii), cnn_cutoff=list(cuts), member_cutoff=5, v=False)
    tree = hierarchy_tree(cl._bundle)
    cl.reel()
    reeled = np.asarray(cl._bundle.labels, dtype=np.int64)
    save("hierarchy_repeat.npz", points=x, radii=radii, cuts=cuts, member_cutoff=np.int64(5), reeled=reeled,
         **tree)


def predict_case(rng):
    centres = np.array([[0.0, 0.0], [2.5, 0.5], [1.0, 2.5]])
    def sample(n):
        return np.vstack([c + rng.normal(0, 0.45, size=(n, 2)) for c in centres] +
                         [rng.uniform(-2, 4.5, size=(n // 5, 2))])
    x = sample(300)
    y = sample(450)
    recipe = {
        "input_data": _types.InputDataExtComponentsMemoryview,
        "fitter": _fit.FitterExtBFS,
        "fitter.ngetter": _types.NeighboursGetterExtBruteForce,
        "fitter.na": _types.NeighboursExtVectorCPPUnorderedSet,
        "fitter.checker": _types.SimilarityCheckerExtSwitchContains,
        "fitter.queue": _types.QueueExtFIFOQueue,
        "fitter.ngetter.dgetter": _types.DistanceGetterExtMetric,
        "fitter.ngetter.dgetter.metric": _types.MetricExtEuclideanReduced,
        "predictor": _fit.PredictorFirstmatch,
        "predictor.ngetter": _types.NeighboursGetterExtBruteForce,
        "predictor.ngetter.dgetter": _types.DistanceGetterExtMetric,
        "predictor.ngetter.dgetter.metric": _types.MetricExtEuclideanReduced,
        "predictor.ogetter": _types.NeighboursGetterExtBruteForce,
        "predictor.ogetter.dgetter": _types.DistanceGetterExtMetric,
        "predictor.ogetter.dgetter.metric": _types.MetricExtEuclideanReduced,
        "predictor.na": _types.NeighboursExtVectorCPPUnorderedSet,
        "predictor.checker": _types.SimilarityCheckerExtSwitchContains,
    }
    out = {"points": x, "other": y}
    for k, (r, c, clusters) in enumerate([(0.3, 4, None), (0.25, 6, [1, 3]), (0.4, 2, None)]):
        cl = cluster.Clustering(np.ascontiguousarray(x), recipe=recipe)
        cl.fit(r, c, member_cutoff=5, v=False)
        other = cluster.Clustering(np.ascontiguousarray(y), recipe=recipe)
        cl.predict(other._bundle, r, c, clusters=clusters)
        out[f"labels_{k}"] = np.asarray(cl.labels, dtype=np.int64)
        out[f"predicted_{k}"] = np.asarray(other._bundle.labels, dtype=np.int64)
        out[f"params_{k}"] = np.array([r, c], dtype=np.float64)
        out[f"clusters_{k}"] = np.array(sorted(clusters) if clusters else [], dtype=np.int64)
    save("predict_firstmatch.npz", n_cases=np.int64(3), **out)


def metric_input_cases(rng):
    # dihedral-like angles in [-180, 180): clusters that wrap around the box
    centres = np.array([[-170.0, 60.0], [175.0, -160.0], [-60.0, -40.0], [60.0, 170.0]])
    ang = np.vstack([c + rng.normal(0, 14.0, size=(700, 2)) for c in centres] +
                    [rng.uniform(-180, 180, size=(300, 2))])
    ang = (ang + 180.0) % 360.0 - 180.0
    ang = ang[rng.permutation(ang.shape[0])]
    bounds = np.array([360.0, 360.0])
    metric = (_types.MetricExtEuclideanPeriodicReduced, (bounds,), {})
    out = {"points": ang, "bounds": bounds}
    for k, (r, c, mc) in enumerate([(10.0, 15, 50), (6.0, 5, 10)]):
        cl = cluster.Clustering(np.ascontiguousarray(ang), fitter__getter__dgetter__metric=metric)
        cl.fit(r, c, member_cutoff=mc, v=False)
        out[f"labels_{k}"] = np.asarray(cl.labels, dtype=np.int64)
        out[f"params_{k}"] = np.array([r, c, mc], dtype=np.float64)
        off, ind = reference_periodic_rows(ang, bounds, r)
        out[f"csr_sha256_{k}"] = np.array(csr_digest(off, ind))
    save("periodic_dihedrals.npz", n_cases=np.int64(2), **out)

    # precomputed distances of a small blob set
    x = np.vstack([c + rng.normal(0, 0.4, size=(250, 2)) for c in ([0, 0], [3, 0], [1.5, 2.5])])
    x = x[rng.permutation(x.shape[0])]
    dist = pairwise_distances(x)
    r, c = 0.35, 5
    cl = cluster.Clustering(np.ascontiguousarray(dist), recipe="distances")
    cl.fit(r, c, member_cutoff=5, v=False)
    square = np.asarray(cl.labels, dtype=np.int64)
    iu = np.triu_indices(x.shape[0], 1)
    lin = np.ascontiguousarray(dist[iu])
    recipe = {"input_data": _types.InputDataExtDistancesLinearMemoryview, "fitter": "bfs",
              "fitter.ngetter": "brute_force", "fitter.na": "vuset", "fitter.checker": "switch",
              "fitter.queue": "fifo", "fitter.ngetter.dgetter": "lookup"}
    cl = cluster.Clustering(_types.InputDataExtDistancesLinearMemoryview(lin), recipe=recipe)
    cl.fit(r, c, member_cutoff=5, v=False)
    linear = np.asarray(cl.labels, dtype=np.int64)
    # the distances are not stored: tests rebuild them with the same expression
    save("precomputed_distances.npz", points=x, radius_cutoff=np.float64(r),
         cnn_cutoff=np.int64(c), member_cutoff=np.int64(5), labels_square=square, labels_linear=linear)


def pairwise_distances(x):
    """Square Euclidean distance matrix (the expression the tests repeat)."""
    return np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))


def reference_periodic_rows(x, bounds, r):
    m = _types.MetricExtEuclideanPeriodicReduced(np.asarray(bounds, dtype=np.float64))
    getter = _types.NeighboursGetterExtBruteForce(_types.DistanceGetterExtMetric(m))
    data = _types.InputDataExtComponentsMemoryview(np.ascontiguousarray(x, dtype=np.float64))
    params = ClusterParameters(r * r)
    nb = _types.NeighboursExtVector(64)
    rows = []
    for i in range(x.shape[0]):
        getter.get(i, data, nb, params)
        rows.append(np.array([nb.get_member(k) for k in range(nb.n_points)], dtype=np.int32))
    offsets = np.zeros(x.shape[0] + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([len(a) for a in rows])
    return offsets, np.concatenate(rows)


def mst_tree(root):
    """Bundles breadth first: path, graph nodes, graph edges (a, b, weight), lambda."""
    from collections import deque
    paths, nodes, edges, lambdas = [], [], [], []
    q = deque([((), root)])
    while q:
        path, b = q.popleft()
        paths.append(".".join(str(p) for p in path))
        g = b._graph
        nodes.append(np.array(sorted(g.nodes), dtype=np.int64) if g is not None else np.zeros(0, dtype=np.int64))
        e = sorted((min(u, v), max(u, v), float(d["weight"])) for u, v, d in g.edges(data=True)) if g is not None \
            else []
        edges.append(np.array(e, dtype=np.float64).reshape(-1, 3))
        lambdas.append(float(b._lambda))
        for label in sorted(b.children):
            q.append((path + (label,), b.children[label]))
    no = np.zeros(len(nodes) + 1, dtype=np.int64)
    no[1:] = np.cumsum([a.shape[0] for a in nodes])
    eo = np.zeros(len(edges) + 1, dtype=np.int64)
    eo[1:] = np.cumsum([a.shape[0] for a in edges])
    return {"paths": np.array(paths), "nodes_off": no, "nodes": np.concatenate(nodes), "edges_off": eo,
            "edges": np.concatenate(edges) if edges else np.zeros((0, 3)), "lambdas": np.array(lambdas)}


def mst_case(rng):
    out = {}
    cases = []
    x1 = np.vstack([c + rng.normal(0, 0.25, size=(150, 2)) for c in ([0, 0], [1.6, 0.2], [0.8, 1.5])] +
                   [rng.uniform(-1, 2.5, size=(40, 2))])
    x1 = x1[rng.permutation(x1.shape[0])]
    cases.append((x1, 0.3, 10))
    x2 = np.vstack([c + rng.normal(0, 0.3, size=(120, 2)) for c in ([0, 0], [4, 4])])  # two components
    cases.append((x2, 0.35, 5))
    for k, (x, r, mc) in enumerate(cases):
        recipe = {"input_data": "components_mview", "preparation_hook": "points_from_parts",
                  "hierarchical_fitter": "mst", "hierarchical_fitter.ngetter": "brute_force",
                  "hierarchical_fitter.ngetter.dgetter": "metric",
                  "hierarchical_fitter.ngetter.dgetter.metric": "euclidean_r",
                  "hierarchical_fitter.na": "vector", "hierarchical_fitter.checker": "screen",
                  "hierarchical_fitter.pq": "maxheap"}
        cl = cluster.Clustering(np.ascontiguousarray(x), recipe=recipe)
        cl.fit_hierarchical(radius_cutoff=r, member_cutoff=mc, v=False)
        tree = mst_tree(cl._bundle)
        out[f"points_{k}"] = x
        out[f"params_{k}"] = np.array([r, mc], dtype=np.float64)
        for key, val in tree.items():
            out[f"{key}_{k}"] = val
    save("mst_prim.npz", n_cases=np.int64(len(cases)), **out)


if __name__ == "__main__":
    main()
