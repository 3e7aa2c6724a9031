"""Which float64 accumulation does the reference's own build use on this host?

Test infrastructure.  The reference sums squared differences with
``total += cpow(a - b, 2)`` (src/cnnclustering/_types.pyx:2253-2267); whether
the compiler fuses that into one FMA depends on the host and the flags.  The
reference's setup.py (setup.py:24-33) builds with the interpreter's
``sysconfig`` CFLAGS minus ``-Wstrict-prototypes`` plus
``-Wno-misleading-indentation -fno-var-tracking-assignments -std=c++14``, as
C++.  ``probe()`` compiles the same loop (``fma_probe_sum.cpp``) with those
flags and the host C++ compiler, links it to a driver built without
contraction, and returns "separate" or "fused" (the library's CNN_FP_SEPARATE
/ CNN_FP_FUSED), or "mixed"/"undecided".
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")


def reference_flags() -> list:
    """The compile flags the reference's setup.py derives on this host."""
    flags = set((sysconfig.get_config_var("CFLAGS") or "").split())
    flags.discard("-Wstrict-prototypes")
    flags.update({"-Wno-misleading-indentation", "-fno-var-tracking-assignments", "-std=c++14"})
    return sorted(flags)


def probe() -> dict:
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    flags = reference_flags()
    obj = os.path.join(OUT_DIR, f"fma_probe_sum.{os.getpid()}.o")
    exe = os.path.join(OUT_DIR, f"fma_probe.{os.getpid()}")
    try:
        subprocess.run([cxx, *flags, "-fPIC", "-c", os.path.join(HERE, "fma_probe_sum.cpp"), "-o", obj], check=True,
                       capture_output=True, text=True)
        subprocess.run([cc, "-O2", "-ffp-contract=off", os.path.join(HERE, "fma_probe_main.c"), obj, "-o", exe, "-lm",
                        "-lstdc++"], check=True, capture_output=True, text=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    finally:
        for p in (obj, exe):
            if os.path.exists(p):
                os.remove(p)
    return {"mode": out[0], "pairs_that_differ": int(out[1]), "matches_separate": int(out[2]),
            "matches_fused": int(out[3]), "compiler": cxx, "flags": flags}


if __name__ == "__main__":
    print(probe())
