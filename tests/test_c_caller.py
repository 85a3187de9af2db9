"""A compiled C caller of the reference's API (tests/c_caller/trafo_adj.c),
built with gcc against include/pnfft.h and libpnfft_gb300.so exactly as
INTEGRATION.md shows: on CPU it must build, link and fail loudly at the first
transform (no GPU, no CPU fallback); on a GPU its trafo and adj results match
the oracle on the same generated inputs (FP64 to 1e-12, FP32-mixed to 1e-6)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_caller", "trafo_adj.c")


def build_caller(lib, tmp_path):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not found")
    libdir = os.path.dirname(lib.build.build())
    exe = str(tmp_path / "trafo_adj")
    cmd = [gcc, "-std=c99", "-Wall", "-Werror", SRC, "-I", os.path.join(ROOT, "include"), "-L", libdir,
           "-lpnfft_gb300", "-Wl,-rpath," + libdir, "-lm", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_c_caller_builds_and_fails_loudly_without_gpu(lib, tmp_path):
    exe = build_caller(lib, tmp_path)
    if lib.device_count() > 0:
        pytest.skip("a GPU is visible: the GPU test runs the caller")
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 4, (r.returncode, r.stderr)  # the trafo reported its error
    assert "CUDA" in r.stderr or "device" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-6)])
def test_c_caller_matches_oracle(lib, oracle, tmp_path, prec, tol):
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    exe = build_caller(lib, tmp_path)
    r = subprocess.run([exe, str(tmp_path), prec], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stderr)
    rd = lambda name: np.fromfile(str(tmp_path / name), dtype=np.float64)  # noqa: E731
    x = rd("x.bin").reshape(-1, 3)
    fh = rd("fhat.bin").view(np.complex128)
    f = rd("f.bin").view(np.complex128)
    adj = rd("adj.bin").view(np.complex128)
    o = oracle.OraclePlan((16, 16, 16), (32, 32, 32), m=4)
    want_f = o.trafo(x, fh)[0]
    want_adj = o.adj(x, f).ravel()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    assert rel(f, want_f) < tol
    assert rel(adj, want_adj) < tol
