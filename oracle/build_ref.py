"""Build recipe for oracle/_ref/libpnfft_ref.so: the reference PNFFT's own C
sources, compiled unmodified from the reference tree against the
single-process stand-ins in oracle/refbuild/ (MPI, PFFT, two GSL functions and
the autotools config.h).  TEST INFRASTRUCTURE ONLY: the tests load it to pin
the oracle to the reference itself; the product never does.

The reference tree is read where it lies (REFERENCE_ROOT, default
/root/reference); nothing is copied.  Without the tree the build is skipped.
-Wl,-Bsymbolic binds the reference's calls to its own functions, so that the
library can share a process with libpnfft_gb300.so (the same pnfft_* names).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SHIM = os.path.join(HERE, "refbuild")
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libpnfft_ref.so")
REF = os.environ.get("REFERENCE_ROOT", "/root/reference")


def sources():
    srcs = sorted(glob.glob(os.path.join(REF, "kernel", "*.c")))
    srcs += sorted(glob.glob(os.path.join(REF, "api", "api-*.c")))
    srcs += sorted(glob.glob(os.path.join(REF, "util", "*.c")))
    srcs += sorted(glob.glob(os.path.join(REF, "cerf", "*.c")))
    return srcs


def available():
    return os.path.isfile(os.path.join(REF, "kernel", "ndft-parallel.c"))


def build(force=False, verbose=False):
    """Compile the reference build if the tree is present; returns the library path or None."""
    if not available():
        return LIB if os.path.exists(LIB) else None
    deps = sources() + glob.glob(os.path.join(SHIM, "*")) + glob.glob(os.path.join(SHIM, "gsl", "*"))
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    obj_dir = os.path.join(OUT_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    inc = ["-I", SHIM, "-I", os.path.join(REF, "kernel"), "-I", os.path.join(REF, "api"), "-I",
           os.path.join(REF, "cerf"), "-I", REF]
    flags = ["-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off", "-w"]
    jobs = []
    for s in sources() + [os.path.join(SHIM, "shim.c")]:
        o = os.path.join(obj_dir, os.path.relpath(s, "/").replace(os.sep, "_") + ".o")
        jobs.append((s, o, [cc, *flags, *inc, "-c", s, "-o", o]))

    def run(job):
        r = subprocess.run(job[2], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("reference build failed:\n" + " ".join(job[2]) + "\n" + r.stderr)
        return job[1]

    with cf.ThreadPoolExecutor(min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(run, jobs))
    r = subprocess.run([cc, "-shared", "-Wl,-Bsymbolic", "-o", LIB + ".tmp", *objs, "-lm"], capture_output=True,
                       text=True)
    if r.returncode:
        raise RuntimeError("reference link failed:\n" + r.stderr)
    shutil.move(LIB + ".tmp", LIB)
    if verbose:
        print(LIB, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
