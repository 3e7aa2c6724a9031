"""Build recipe for the oracle's C restatement (test infrastructure only).

Compiles ``oracle/cnn_oracle.c`` with the host C compiler into
``oracle/_build/libcnn_oracle.so``.  ``-ffp-contract=off`` keeps the
compiler from fusing the multiply-add of the distance sum, so the
floating-point mode is exactly the one the caller selects.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cnn_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcnn_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [os.environ.get("CC", "gcc"), "-O2", "-ffp-contract=off", "-fPIC", "-shared",
           "-Wall", "-o", tmp, SRC, "-lm", "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
