"""Builds libpnfft_gb300.so in-tree (pnfft_gb300/libpnfft_gb300.so).

nvcc compiles the CUDA sources for sm_103a only (one -gencode) and g++ the
host C ABI; translation units are compiled in parallel.  Object files go to
pnfft_gb300/_build/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpnfft_gb300.so")
INC = os.path.join(os.path.dirname(HERE), "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["conv.cu", "float_io.cu", "interp_line.cu", "interp_line_g.cu", "spread_line_f.cu", "interp_group.cu", "interp_tile_f32.cu", "interp_tile_f64.cu", "spread_line_f32.cu",
              "spread_line_f64.cu", "generic.cu", "deconv.cu", "sort.cu", "ndft.cu", "engine.cu", "peak.cu"]
CPP_SOURCES = ["api.cpp", "api_float.cpp"]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INC, f) for f in os.listdir(INC)]
    return files


def _up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force=False, verbose=False, jobs=None):
    """Compile the library if any source changed; returns its path."""
    if not force and _up_to_date():
        return LIB
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(OBJ, exist_ok=True)
    common = ["-O3", "-std=c++17", "-I", CSRC, "-I", INC]
    cmds = []
    for s in CU_SOURCES:
        o = os.path.join(OBJ, s + ".o")
        cmds.append([NVCC, *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", *common, "-c",
                     os.path.join(CSRC, s), "-o", o])
    for s in CPP_SOURCES:
        o = os.path.join(OBJ, s + ".o")
        cmds.append(["g++", "-fPIC", "-Wall", "-Wno-unused-function", "-ffp-contract=off", *common, "-I",
                     os.path.join(CUDA_HOME, "include"), "-c", os.path.join(CSRC, s), "-o", o])
    jobs = jobs or min(len(cmds), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose:
        for c, o in zip(cmds, outs):
            print(" ".join(c), file=sys.stderr)
            if o.strip():
                print(o, file=sys.stderr)
    objs = [os.path.join(OBJ, s + ".o") for s in CU_SOURCES + CPP_SOURCES]
    tmp = LIB + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcufft", "-Xlinker",
          "-rpath," + os.path.join(CUDA_HOME, "lib64")])
    shutil.move(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
