"""CPU checks of the C-ABI library: it builds, loads, and exports every
entry point include/cnngpu.h declares.  No compute call is made here."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "cnngpu.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"CNN_API\s+[\w\s\*]+?\b(cnn_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path():
    from commonnnclustering_gb300 import _build
    return _build.build()


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "cnn_fit" in syms and "cnn_build_neighbours" in syms and "cnn_sort_by_size" in syms
    assert len(syms) >= 15


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True)
    exported = set(line.split()[-1] for line in out.stdout.splitlines() if " T " in line)
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_library_loads_and_reports_abi_version(lib_path):
    L = ctypes.CDLL(lib_path)
    for s in declared_symbols():
        assert hasattr(L, s), s
    assert L.cnn_abi_version() == 2


def test_python_binding_covers_header():
    from commonnnclustering_gb300 import _abi
    assert sorted(_abi.SIGNATURES) == declared_symbols()


def test_build_targets_sm_103a_only():
    from commonnnclustering_gb300 import _build
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_binding_abi_version_is_the_headers():
    """The ctypes structs mirror one version of include/cnngpu.h; the binding
    refuses a library of another version at load time."""
    from commonnnclustering_gb300 import _abi
    hdr = open(HEADER).read()
    m = re.search(r"#define CNN_ABI_VERSION (\d+)", hdr)
    assert m and int(m.group(1)) == _abi.ABI_VERSION
