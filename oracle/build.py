"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/pnfft_oracle.c into oracle/_build/liboracle.so with gcc.
`-ffp-contract=off` keeps gcc from fusing a*b+c into an FMA (the default on
aarch64), so that floor(n*x - m) and friends round exactly like the
reference's x86-64 build, which has no FMA in its baseline ISA.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "pnfft_oracle.c")


def _needs_build():
    if not os.path.exists(LIB):
        return True
    return os.path.getmtime(LIB) < os.path.getmtime(SRC)


def build(force=False, verbose=False):
    """Compile the oracle if needed; returns the path of the shared library."""
    if not force and not _needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    base = [cc, "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", SRC, "-o", LIB + ".tmp", "-lm"]
    cmd = base[:3] + ["-fopenmp"] + base[3:]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        # no OpenMP runtime: build the serial oracle
        res = subprocess.run(base, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    shutil.move(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
