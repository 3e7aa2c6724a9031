"""Seeded synthetic inputs with the shapes of the benchmark workloads.

No dataset is downloaded; each generator draws from numpy's default_rng
with a fixed seed, so the same call gives the same points everywhere.

* ``blobs2d``   -- 5,000 x 2 float64: three isotropic Gaussians (std 0.5,
  centres uniform in [-5, 5]^2 from seed 0, weights 0.40/0.35/0.15) plus
  10 % uniform noise over [-7, 7]^2.  Fit at r=0.3, c=5, member_cutoff=10.
* ``md3d``      -- 200,000 x 3 float64: 20 anisotropic Gaussians
  (random rotation x diag stds in [0.05, 0.4], Dirichlet(1) weights) plus
  5 % uniform background in the bounding box.  Fit at r=0.1, c=10,
  member_cutoff=50.  Centres are spread so the mean degree is about 200.
* ``features``  -- n x 64 float64: 50 Gaussian clusters (std 0.3, centres
  N(0, 2^2 I)) plus rank-8 correlated noise.
* ``nested3d``  -- n x 3 float32: 100 parent Gaussians (std 0.5), each with
  4 children (std 0.05).
"""
from __future__ import annotations

import numpy as np


def blobs2d(n: int = 5000, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-5.0, 5.0, size=(3, 2))
    weights = np.array([0.40, 0.35, 0.15])
    counts = np.floor(weights * n).astype(int)
    n_noise = n - int(counts.sum())
    parts = [rng.normal(loc=c, scale=0.5, size=(k, 2)) for c, k in zip(centres, counts)]
    parts.append(rng.uniform(-7.0, 7.0, size=(n_noise, 2)))
    x = np.vstack(parts)
    return np.ascontiguousarray(x[rng.permutation(n)], dtype=np.float64)


def _random_rotation(rng, d):
    q, r = np.linalg.qr(rng.normal(size=(d, d)))
    return q * np.sign(np.diag(r))


def md3d(n: int = 200_000, seed: int = 3, n_components: int = 20,
         centre_spread: float = 3.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    weights = rng.dirichlet(np.ones(n_components))
    n_bg = int(round(0.05 * n))
    counts = rng.multinomial(n - n_bg, weights)
    centres = rng.uniform(-centre_spread, centre_spread, size=(n_components, 3))
    parts = []
    for c, k in zip(centres, counts):
        rot = _random_rotation(rng, 3)
        stds = rng.uniform(0.05, 0.4, size=3)
        z = rng.normal(size=(k, 3)) * stds
        parts.append(c + z @ rot.T)
    x = np.vstack(parts)
    lo, hi = x.min(axis=0), x.max(axis=0)
    parts.append(rng.uniform(lo, hi, size=(n_bg, 3)))
    x = np.vstack(parts)
    return np.ascontiguousarray(x[rng.permutation(n)], dtype=np.float64)


def features(n: int = 500_000, d: int = 64, seed: int = 2, n_clusters: int = 50,
             noise_rank: int = 8, noise_scale: float = 0.3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    centres = rng.normal(0.0, 2.0, size=(n_clusters, d))
    assign = rng.integers(0, n_clusters, size=n)
    x = centres[assign] + rng.normal(0.0, 0.3, size=(n, d))
    basis = rng.normal(size=(noise_rank, d)) / np.sqrt(d)
    x += noise_scale * rng.normal(size=(n, noise_rank)) @ basis
    return np.ascontiguousarray(x, dtype=np.float64)


def nested3d(n: int = 1_000_000, seed: int = 3, n_parents: int = 100,
             children: int = 4, box: float = 20.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parents = rng.uniform(-box, box, size=(n_parents, 3))
    kids = parents[:, None, :] + rng.normal(0.0, 0.5, size=(n_parents, children, 3))
    kids = kids.reshape(-1, 3)
    which = rng.integers(0, kids.shape[0], size=n)
    x = kids[which] + rng.normal(0.0, 0.05, size=(n, 3))
    return np.ascontiguousarray(x, dtype=np.float32)


def mixture(n: int, d: int, n_components: int, seed: int, noise: float = 0.05) -> np.ndarray:
    """Gaussian mixture (unit within-component std) plus uniform noise in its box."""
    rng = np.random.default_rng(seed)
    spread = 6.0 * max(1.0, n_components ** (1.0 / d)) if d <= 3 else 4.0
    centres = rng.uniform(-spread, spread, size=(n_components, d)) if d <= 3 else \
        rng.normal(0.0, spread, size=(n_components, d))
    n_noise = int(round(noise * n))
    counts = rng.multinomial(n - n_noise, rng.dirichlet(np.ones(n_components)))
    x = np.vstack([c + rng.normal(size=(k, d)) for c, k in zip(centres, counts)])
    lo, hi = x.min(axis=0), x.max(axis=0)
    x = np.vstack([x, rng.uniform(lo, hi, size=(n_noise, d))])
    return np.ascontiguousarray(x[rng.permutation(n)], dtype=np.float64)


def degree_radius(x: np.ndarray, degree, seed: int = 0, queries: int = 96, max_sample: int = 10000):
    """Radius giving about `degree` neighbours per point (sampled estimate).

    ``degree`` may be a sequence: then one radius per target, from one set
    of sampled squared distances."""
    many = np.ndim(degree) > 0
    degrees = np.atleast_1d(np.asarray(degree, dtype=np.float64))
    rng = np.random.default_rng(seed)
    n = x.shape[0]
    m = min(n, max_sample)
    sample = x[rng.choice(n, m, replace=False)] if m < n else x
    q = x[rng.choice(n, min(queries, n), replace=False)]
    d2 = (q * q).sum(1)[:, None] + (sample * sample).sum(1)[None] - 2.0 * q @ sample.T
    ks = [max(2, int(round(deg * m / n))) for deg in degrees]
    kth = np.partition(d2, sorted({min(k, m - 1) for k in ks}), axis=1)
    out = []
    for deg, k in zip(degrees, ks):
        r = float(np.sqrt(max(np.median(kth[:, min(k, m - 1)]), 1e-12)))
        if k > deg * m / n:  # the sample was too small for the target: shrink by volume
            r *= (deg * m / n / k) ** (1.0 / x.shape[1])
        out.append(r)
    return out if many else out[0]


def job_stream(n_jobs: int = 2000, rate: float = 100.0, seed: int = 11, pool=None, max_points=2_000_000):
    """Served workload: Poisson arrivals of clustering jobs.

    Point counts lognormal (median 20k, sigma 1.2) clipped to [1k,
    max_points = 2M]; d from {2, 3, 16, 64}; each job its own Gaussian
    mixture of 5-200 components + 5 % uniform noise, its own radius (tuned
    for a mean degree drawn from [50, 300]) and cnn_cutoff in [3, 50];
    member_cutoff 10.  ``pool``: draw the jobs' points from that many shared
    datasets instead (faster to generate; each job keeps its own degree
    target and cnn_cutoff).  Returns a list of dicts: arrival, points,
    radius_cutoff, cnn_cutoff, member_cutoff, expected_degree.
    """
    rng = np.random.default_rng(seed)

    def dataset(k: int):
        d = int(rng.choice([2, 3, 16, 64]))
        n = int(np.clip(np.exp(rng.normal(np.log(20000.0), 1.2)), 1000, max_points))
        comps = int(rng.integers(5, 201))
        x = mixture(n, d, comps, seed=seed * 100003 + k)
        radii = dict(zip((50, 100, 200, 300), degree_radius(x, (50, 100, 200, 300), seed=k)))
        return x, radii

    datasets = [dataset(p) for p in range(pool)] if pool else None
    t = 0.0
    jobs = []
    for i in range(n_jobs):
        t += rng.exponential(1.0 / rate)
        x, radii = datasets[int(rng.integers(0, pool))] if pool else dataset(i)
        deg = float(rng.uniform(50, 300))
        keys = sorted(radii)
        r = float(np.interp(deg, keys, [radii[k] for k in keys]))
        jobs.append(dict(arrival=t, points=x, radius_cutoff=r, cnn_cutoff=int(rng.integers(3, 51)),
                         member_cutoff=10, expected_degree=deg * 1.5))
    return jobs


WORKLOADS = {
    "blobs2d-5k": dict(gen=blobs2d, n=5000, radius_cutoff=0.3, cnn_cutoff=5, member_cutoff=10),
    "md3d-200k": dict(gen=md3d, n=200_000, radius_cutoff=0.1, cnn_cutoff=10, member_cutoff=50),
}
