"""Per-plan autotuning (pnfft_gb300_autotune, pnfft_gb300_get_tuning /
pnfft_gb300_set_tuning) on the GPU.

The autotuner only chooses among kernels that each pass the parity tests, so
what is checked here is that it runs on host and device arrays, returns a
valid tuning, leaves the caller's arrays alone, and that transforms after it
still match the oracle within the FP32-mixed tolerance (1e-6 relative l2);
and that a tuning set by hand is the one the next call uses.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    d = np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel())
    nb = np.linalg.norm(np.asarray(b).ravel())
    return d / nb if nb > 0 else d


@pytest.fixture(scope="module")
def gpu(lib):
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    return lib


def clustered(rng, M):
    x = rng.uniform(-0.5, 0.5, (M, 3))
    c = rng.uniform(-0.5, 0.5, (8, 3))
    k = M // 3
    x[:k] = c[rng.integers(0, 8, k)] + 0.01 * rng.standard_normal((k, 3))
    return np.mod(x + 0.5, 1.0) - 0.5


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("grad", [False, True])
def test_autotune_device_then_parity(gpu, oracle, prec, grad):
    import torch
    N, m, M = (16, 16, 16), 5, 6000
    rng = np.random.default_rng(41)
    x = clustered(rng, M)
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    p = gpu.Plan(N, m=m, precision=prec)
    o = oracle.OraclePlan(N, m=m)
    tflags = gpu.COMPUTE_F | (gpu.COMPUTE_GRAD_F if grad else 0)
    xd = torch.tensor(x, device="cuda")
    fhd = torch.tensor(fh.ravel(), device="cuda")
    fh_keep = fhd.clone()
    t = p.autotune_device(xd, fhd, tflags, gpu.COMPUTE_F, reps=1)
    assert torch.equal(fhd, fh_keep)
    assert len(t) == 3 and t[2] in (256, 512, 2048)
    if prec == "fp64":
        assert t[:2] == (0, 0)  # one family per direction in FP64
    else:
        assert t[0] in (0, 2) and t[1] in (0, 2)
    tol = 1e-6 if prec == "fp32" else 1e-12
    ref_f, ref_g, _ = o.trafo(x, fh, tflags)
    got_f, got_g, _ = p.trafo_device(xd, fhd, tflags)
    assert rel(got_f.cpu().numpy(), ref_f) < tol
    if grad:
        assert rel(got_g.cpu().numpy(), ref_g) < tol
    got = p.adj_device(xd, torch.tensor(f, device="cuda"))
    assert rel(got.cpu().numpy(), o.adj(x, f).ravel()) < tol
    p.close()


def test_autotune_host_arrays_and_set_tuning(gpu, oracle):
    """The C entry on host arrays, then each hand-set tuning in turn."""
    L = gpu.load()
    N, m, M = (16, 16, 16), 4, 5000
    rng = np.random.default_rng(42)
    x = clustered(rng, M)
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    p = gpu.Plan(N, m=m, precision="fp32")
    o = oracle.OraclePlan(N, m=m)
    ref = o.trafo(x, fh, gpu.COMPUTE_F)[0]
    # host arrays of the plan's nodes, alive through the C call
    xh = np.ascontiguousarray(x)
    fo = np.zeros(M, np.complex128)
    fhh = fh.ravel().copy()  # the adjoint of the autotuner writes its f_hat here
    nd = p._nodes_for(M)
    L.pnfft_set_x(xh.ctypes.data, nd)
    L.pnfft_set_f(fo.ctypes.data, nd)
    L.pnfft_set_grad_f(None, nd)
    L.pnfft_set_hessian_f(None, nd)
    L.pnfft_set_f_hat(fhh.ctypes.data, p._p)
    L.pnfft_gb300_clear_error()
    rc = L.pnfft_gb300_autotune(p._p, nd, ctypes.c_uint(gpu.COMPUTE_F), ctypes.c_uint(gpu.COMPUTE_F), 1)
    gpu._check(rc, "pnfft_gb300_autotune")
    assert rel(p.trafo(x, fh)[0], ref) < 1e-6
    for t in [(0, 0, 256), (2, 2, 512), (0, 2, 2048), (2, 0, 512), (1, 1, 512)]:
        p.set_tuning(t)
        assert p.tuning() == t
        assert rel(p.trafo(x, fh)[0], ref) < 1e-6
    with pytest.raises(gpu.PnfftError):
        p.set_tuning((0, 0, 100))
    p.close()
