"""Which float64 accumulation the reference's own build reproduces.

The reference's distance loop (src/cnnclustering/_types.pyx:2253-2267) is
compiled with its setup.py flags (-std=c++14 among them) by the host's C++
compiler; oracle/fma_probe.py builds the same loop with those flags and
reports whether it fuses the multiply-add.  The library's default fpmode
(CNN_FP_SEPARATE) must be the one the reference reproduces: on this
container (x86-64, where the golden fixtures were made) and on the GB300
host (aarch64), which the gpu-marked copy of the check runs on.
"""
import shutil

import pytest


def _probe():
    if not (shutil.which("g++") and shutil.which("gcc")):
        pytest.skip("no host C/C++ compiler")
    from oracle import fma_probe
    return fma_probe.probe()


def test_reference_build_accumulates_separately_here():
    r = _probe()
    assert r["pairs_that_differ"] > 1000
    assert r["mode"] == "separate", r


@pytest.mark.gpu
def test_reference_build_accumulates_separately_on_the_gpu_host():
    """Runs where the GPU tests run (the GB300's aarch64 host)."""
    import platform
    r = _probe()
    print(f"{platform.machine()}: reference build flags {r['flags']} -> {r['mode']}")
    assert r["pairs_that_differ"] > 1000
    assert r["mode"] == "separate", r
