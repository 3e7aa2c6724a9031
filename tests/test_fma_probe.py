"""Which float64 accumulation the reference's own build reproduces, and
that the library's default follows it.

The reference's distance loop (src/cnnclustering/_types.pyx:2253-2267) is
compiled with its setup.py flags (-std=c++14 among them) by the host's C++
compiler; oracle/fma_probe.py builds the same loop with those flags and
reports whether it fuses the multiply-add.  Measured: x86-64 keeps two
roundings ("separate"), the GB300's aarch64 host fuses ("fused").  The
library's default fpmode ("auto", ``_abi.host_fpmode``) must be the mode the
probe reports on the host it runs on: the CPU test checks this container,
the gpu-marked copy the GPU host.
"""
import shutil

import numpy as np
import pytest


def _probe():
    if not (shutil.which("g++") and shutil.which("gcc")):
        pytest.skip("no host C/C++ compiler")
    from oracle import fma_probe
    return fma_probe.probe()


def _library_default(monkeypatch):
    monkeypatch.delenv("CNN_FPMODE", raising=False)
    from commonnnclustering_gb300 import _abi
    return "fused" if _abi.host_fpmode() == _abi.FP_FUSED else "separate"


def test_library_default_is_the_reference_build_mode_here(monkeypatch):
    r = _probe()
    assert r["pairs_that_differ"] > 1000
    assert r["mode"] in ("separate", "fused"), r
    assert _library_default(monkeypatch) == r["mode"]


@pytest.mark.gpu
def test_library_default_is_the_reference_build_mode_on_the_gpu_host(monkeypatch):
    """Runs where the GPU tests run (the GB300's aarch64 host); the default
    Clustering then equals the oracle in that mode."""
    import platform
    r = _probe()
    print(f"{platform.machine()}: reference build flags {r['flags']} -> {r['mode']}")
    assert r["pairs_that_differ"] > 1000
    mode = _library_default(monkeypatch)
    assert mode == r["mode"], r
    import commonnnclustering_gb300 as cnn
    from commonnnclustering_gb300 import workloads
    from oracle import cnn_oracle
    x = workloads.md3d(n=30000, seed=12, centre_spread=2.0)
    cl = cnn.Clustering(x)
    cl.fit(0.1, 8, member_cutoff=10, v=False)
    want, info = cnn_oracle.clustering_fit(x, 0.1, 8, member_cutoff=10,
                                          fpmode=cnn_oracle.FP_FUSED if mode == "fused" else cnn_oracle.FP_SEPARATE)
    assert np.array_equal(np.asarray(cl.labels), want)
