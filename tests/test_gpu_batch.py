"""Batches of uneven plans and shared-node right-hand sides replayed as one
CUDA graph (pnfft_gb300.batch): the replay reproduces the eager calls, follows
in-place changes of the inputs, matches the oracle, and host arrays are
refused while a stream is being captured."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_batch_graph_replays_eager_results(lib, oracle):
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    from pnfft_gb300.batch import Batch
    rng = np.random.default_rng(51)
    dev = "cuda"
    specs = [((16, 16, 16), 3000, 4, "fp32"), ((16, 32, 48), 500, 5, "fp32"), ((32, 32, 32), 20000, 6, "fp32"),
             ((16, 16, 32), 700, 4, "fp64")]
    batch = Batch()
    outs = []
    for N, M, m, prec in specs:
        p = lib.Plan(N, m=m, precision=prec)
        x = torch.tensor(rng.uniform(-0.5, 0.5, (M, 3)), device=dev)
        S = int(np.prod(N))
        fh = torch.tensor(rng.standard_normal(S) + 1j * rng.standard_normal(S), device=dev)
        f_in = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), device=dev)
        f_out = torch.empty(M, dtype=torch.complex128, device=dev)
        fh_out = torch.empty(S, dtype=torch.complex128, device=dev)
        batch.add_trafo(p, x, fh, f_out)
        batch.add_adj(p, x, f_in, fh_out)
        outs.append((p, N, m, prec, x, fh, f_in, f_out, fh_out))
    # K = 3 right-hand sides sharing one node set
    pk = lib.Plan((16, 16, 16), m=5, precision="fp32")
    xk = torch.tensor(rng.uniform(-0.5, 0.5, (4000, 3)), device=dev)
    rhs = []
    for _ in range(3):
        fh = torch.tensor(rng.standard_normal(4096) + 1j * rng.standard_normal(4096), device=dev)
        fo = torch.empty(4000, dtype=torch.complex128, device=dev)
        batch.add_trafo(pk, xk, fh, fo)
        rhs.append((fh, fo))
    batch.run_eager()
    batch.synchronize()
    eager = [(o[7].clone(), o[8].clone()) for o in outs] + [fo.clone() for _, fo in rhs]
    batch.autotune(reps=1)
    batch.capture()
    for o in outs:
        o[7].zero_()
        o[8].zero_()
    batch.run()
    batch.synchronize()
    for (p, N, m, prec, *_), o, e in zip(outs, outs, eager):
        tol = 1e-12 if prec == "fp64" else 1e-5  # the autotuner may pick the other kernels
        assert _rel(o[7].cpu().numpy(), e[0].cpu().numpy()) < tol
        assert _rel(o[8].cpu().numpy(), e[1].cpu().numpy()) < tol
    for (fh, fo), e in zip(rhs, eager[len(outs):]):
        assert _rel(fo.cpu().numpy(), e.cpu().numpy()) < 1e-5
    # the graph reads the inputs in place: a new right-hand side gives its transform
    fh_new = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
    rhs[0][0].copy_(torch.tensor(fh_new, device=dev))
    batch.run()
    batch.synchronize()
    o = oracle.OraclePlan((16, 16, 16), m=5)
    want = o.trafo(xk.cpu().numpy(), fh_new)[0]
    assert _rel(rhs[0][1].cpu().numpy(), want) < 1e-6
    # the FP64 plan against the oracle
    p, N, m, prec, x, fh, f_in, f_out, fh_out = outs[3]
    o = oracle.OraclePlan(N, m=m)
    assert _rel(f_out.cpu().numpy(), o.trafo(x.cpu().numpy(), fh.cpu().numpy())[0]) < 1e-12
    assert _rel(fh_out.cpu().numpy(), o.adj(x.cpu().numpy(), f_in.cpu().numpy())) < 1e-12


def test_capture_refuses_host_arrays(lib):
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    L = lib.load()
    p = lib.Plan((8, 8, 8), m=3, precision="fp32")
    x = np.random.default_rng(52).uniform(-0.5, 0.5, (50, 3))
    fh = np.ones(512, complex)
    p.trafo(x, fh)  # warm-up on host arrays
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
        L.pnfft_gb300_set_stream(p.handle, torch.cuda.current_stream().cuda_stream)
        with pytest.raises(lib.PnfftError, match="captured into a CUDA graph"):
            p.trafo(x, fh)
    L.pnfft_gb300_set_stream(p.handle, None)
    f, _, _ = p.trafo(x, fh)  # the plan still works afterwards
    assert np.isfinite(f).all()
