"""bench.py's roofline entry on CPU: the dominant stage, its algorithmic
bytes or flops, and the fields the JSON line carries."""
import pytest


@pytest.fixture()
def bench():
    import bench as b
    return b


def stats(**ms):
    base = {k: 0.0 for k in ("ms_bbox", "ms_cells", "ms_count", "ms_scan", "ms_fill", "ms_nodes", "ms_check",
                             "ms_label", "ms_sort", "ms_gram")}
    base.update(ms)
    base["n_candidates"] = 1 << 20
    return base


def test_hbm_entry_takes_the_slowest_stage(bench):
    n, nnz = 200_000, 43_000_000
    s = [stats(ms_count=0.30, ms_check=0.35, ms_fill=0.08), stats(ms_count=0.32, ms_check=0.33, ms_fill=0.08)]
    e = bench.hbm_roofline(s, nnz, n, {"hbm_gbs": 7000.0})
    assert e["bound"] == "hbm" and e["unit"] == "GB/s" and e["kernel"] == "check_union_kernel"
    assert e["ms_per_launch"] == pytest.approx(0.34)
    want_bytes = 4 * nnz + 8 * (n + 1) + n + 8 * n
    assert e["algorithmic_bytes"] == want_bytes
    assert e["achieved"] == pytest.approx(want_bytes / 0.34e-3 / 1e9)
    assert e["frac"] == pytest.approx(e["achieved"] / 7000.0)
    assert set(e) >= {"bound", "achieved", "peak", "unit", "frac", "traffic"}


def test_tensor_entry_counts_the_issued_mmas(bench):
    s = [stats(ms_gram=2.0, ms_count=5.0)]
    e = bench.tensor_roofline(bench.WORKLOADS["features-500k-d64"], s, 500_000, {"bf16_tflops": 2000.0})
    useful = 2.0 * (1 << 20) * 64
    assert e["bound"] == "tensor" and e["unit"] == "TFLOP/s"
    assert e["algorithmic_flops_issued"] == pytest.approx(6 * useful)
    assert e["achieved"] == pytest.approx(6 * useful / 2.0e-3 / 1e12)
    assert e["frac"] == pytest.approx(e["achieved"] / 2000.0)


def test_default_run_covers_every_workload(bench):
    """bench.py without arguments measures the headline and the four other
    workloads (sub-records of the same JSON line)."""
    assert bench.HEADLINE == "md3d-200k"
    names = {bench.WORKLOADS[w]["name"] for w in bench.SUB_WORKLOADS}
    assert names == {"blobs2d-5k", "features-500k-d64", "nested3d-1m-sweep", "serve-stream"}
