"""The reference-side binding (a Cython module a cnnclustering maintainer
adds, commonnnclustering_gb300/reference_binding/_gpu.pyx) compiles against
include/cnngpu.h and the reference's own .pxd files, links libcnngpu.so, and
registers as one of the reference's Fitters -- checked here without a GPU
(the context is created at the first fit)."""
import os
import subprocess
import sys
import sysconfig

import numpy as np
import pytest

from conftest import ROOT

REF = os.path.join(ROOT, "baseline", "_ref")
PYX = os.path.join(ROOT, "commonnnclustering_gb300", "reference_binding", "_gpu.pyx")


@pytest.fixture(scope="module")
def gpu_module(tmp_path_factory):
    if not os.path.isdir(os.path.join(REF, "cnnclustering")):
        pytest.skip("reference package not installed here")
    pytest.importorskip("Cython")
    from Cython.Build import cythonize
    from commonnnclustering_gb300 import _abi, _build
    _abi.load()  # builds libcnngpu.so when missing
    out = tmp_path_factory.mktemp("binding")
    src = out / "_gpu.pyx"
    src.write_text(open(PYX).read())
    sys.path.insert(0, REF)
    try:
        cythonize([str(src)], include_path=[REF, np.get_include()], quiet=True, language_level=3)
        assert (out / "_gpu.cpp").exists()  # C++ mode: the reference's .pxd files use libcpp
        so = out / ("_gpu" + sysconfig.get_config_var("EXT_SUFFIX"))
        lib_dir = os.path.dirname(_build.LIB)
        cmd = ["g++", "-shared", "-fPIC", "-O1", "-w", str(out / "_gpu.cpp"), "-o", str(so),
               "-I", sysconfig.get_paths()["include"], "-I", np.get_include(), "-I", os.path.join(ROOT, "include"),
               "-L", lib_dir, "-lcnngpu", f"-Wl,-rpath,{lib_dir}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        sys.path.insert(0, str(out))
        import importlib
        mod = importlib.import_module("_gpu")
        yield mod
    finally:
        for p in (str(out), REF):
            if p in sys.path:
                sys.path.remove(p)


def test_binding_is_a_reference_fitter(gpu_module):
    from cnnclustering import _fit, cluster
    assert issubclass(gpu_module.FitterExtGPU, _fit.FitterExtInterface)
    x = np.random.default_rng(0).random((50, 2))
    cl = cluster.Clustering(x)  # the default recipe: brute force, reduced Euclidean, self-counting
    f = gpu_module.FitterExtGPU(cl._fitter._neighbours_getter)
    assert isinstance(f, _fit.Fitter)
    # make_parameters is the reference's own (src/cnnclustering/_fit.pyx:130-161)
    p = f.make_parameters(0.5, 3, 1)
    assert p.radius_cutoff == 0.25 and p.n_member_cutoff == 4 and p.similarity_cutoff == 5
    cl._fitter = f  # the drop-in: Clustering.fit now reaches FitterExtGPU.fit
    assert cl._fitter is f
