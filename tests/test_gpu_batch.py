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


def test_fused_batch_matches_separate_calls(lib, oracle):
    """pnfft_gb300_batch_begin / _end (Batch(fused=True)): the f-only FP32
    line convolutions of plans with cutoffs 9, 11 and 13 and of 3 right-hand
    sides on one node set run as one launch per direction and cutoff; the
    FP64 plan and the gradient trafo run as usual inside the same batch.
    Interpolation results equal the separate calls bit for bit (a node's sum
    has a fixed order); spreading results agree to FP32 rounding, and both
    match the oracle.  The captured graph of the fused batch replays them."""
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    from pnfft_gb300.batch import Batch
    rng = np.random.default_rng(61)
    dev = "cuda"
    specs = [((16, 16, 16), 3000, 4, "fp32"), ((16, 32, 16), 800, 5, "fp32"), ((32, 32, 32), 20000, 6, "fp32"),
             ((16, 16, 16), 700, 4, "fp64")]
    batch = Batch(fused=True)
    ref = []
    for N, M, m, prec in specs:
        p = lib.Plan(N, m=m, precision=prec)
        x = torch.tensor(rng.uniform(-0.5, 0.5, (M, 3)), device=dev)
        S = int(np.prod(N))
        fh = torch.tensor(rng.standard_normal(S) + 1j * rng.standard_normal(S), device=dev)
        f_in = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), device=dev)
        f_out = torch.zeros(M, dtype=torch.complex128, device=dev)
        fh_out = torch.zeros(S, dtype=torch.complex128, device=dev)
        batch.add_trafo(p, x, fh, f_out)
        batch.add_adj(p, x, f_in, fh_out)
        ref.append((p, N, m, prec, x, fh, f_in, f_out, fh_out))
    # a gradient trafo (not deferred) and K = 3 right-hand sides on one node set
    pg = lib.Plan((16, 16, 16), m=5, precision="fp32")
    xg = torch.tensor(rng.uniform(-0.5, 0.5, (1500, 3)), device=dev)
    fhg = torch.tensor(rng.standard_normal(4096) + 1j * rng.standard_normal(4096), device=dev)
    fg = torch.zeros(1500, dtype=torch.complex128, device=dev)
    gg = torch.zeros(1500, 3, dtype=torch.complex128, device=dev)
    batch.add_trafo(pg, xg, fhg, fg, lib.COMPUTE_F | lib.COMPUTE_GRAD_F, grad=gg)
    pk = lib.Plan((16, 16, 16), m=6, precision="fp32")
    xk = torch.tensor(rng.uniform(-0.5, 0.5, (4000, 3)), device=dev)
    rhs = []
    for _ in range(3):
        fh = torch.tensor(rng.standard_normal(4096) + 1j * rng.standard_normal(4096), device=dev)
        fo = torch.zeros(4000, dtype=torch.complex128, device=dev)
        batch.add_trafo(pk, xk, fh, fo)
        rhs.append((fh, fo))
    batch.run_eager()
    batch.synchronize()
    deferred, launches = batch.fused_stats()
    assert deferred == 3 * 2 + 3  # three FP32 plans x (trafo, adj) + the three right-hand sides
    assert launches == 3 + 3      # cutoffs 9, 11, 13 for B; 9, 11, 13 for B^T
    # the same calls one by one, outside any batch
    for p, N, m, prec, x, fh, f_in, f_out, fh_out in ref:
        f_sep, _, _ = p.trafo_device(x, fh, lib.COMPUTE_F)
        fh_sep = p.adj_device(x, f_in)
        torch.cuda.synchronize()
        o = oracle.OraclePlan(N, m=m)
        xs = x.cpu().numpy()
        if prec == "fp32":
            assert torch.equal(f_out, f_sep)
            assert _rel(fh_out.cpu().numpy(), fh_sep.cpu().numpy()) < 1e-6
            tol = 1e-6
        else:
            tol = 1e-12
        assert _rel(f_out.cpu().numpy(), o.trafo(xs, fh.cpu().numpy())[0]) < tol
        assert _rel(fh_out.cpu().numpy(), o.adj(xs, f_in.cpu().numpy()).ravel()) < tol
    f_sep, g_sep, _ = pg.trafo_device(xg, fhg, lib.COMPUTE_F | lib.COMPUTE_GRAD_F)
    torch.cuda.synchronize()
    assert torch.equal(fg, f_sep) and torch.equal(gg, g_sep)
    ok = oracle.OraclePlan((16, 16, 16), m=6)
    for fh, fo in rhs:
        f_sep, _, _ = pk.trafo_device(xk, fh, lib.COMPUTE_F)
        torch.cuda.synchronize()
        assert torch.equal(fo, f_sep)
        assert _rel(fo.cpu().numpy(), ok.trafo(xk.cpu().numpy(), fh.cpu().numpy())[0]) < 1e-6
    # the captured graph of the fused batch
    want = [(r[7].clone(), r[8].clone()) for r in ref] + [fo.clone() for _, fo in rhs]
    batch.capture()
    for r in ref:
        r[7].zero_()
        r[8].zero_()
    for _, fo in rhs:
        fo.zero_()
    batch.run()
    batch.synchronize()
    for r, (wf, wa) in zip(ref, want):
        assert torch.equal(r[7], wf)
        assert _rel(r[8].cpu().numpy(), wa.cpu().numpy()) < 1e-6
    for (_, fo), w in zip(rhs, want[len(ref):]):
        assert torch.equal(fo, w)


def test_batch_rebinning_and_accumulated_adjoint(lib, oracle):
    """Inside one pnfft_gb300 batch: a second trafo on the plan's node set with
    new coordinates rebins the set, so the batch runs the first deferred call
    before (two batched launches); an adjoint with COMPUTE_ACCUMULATED adds to
    f_hat.  Results equal the separate calls (B bit for bit) and the oracle."""
    import ctypes
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    L = lib.load()
    rng = np.random.default_rng(62)
    N, m, M = (16, 16, 16), 5, 3000
    p = lib.Plan(N, m=m, precision="fp32")
    o = oracle.OraclePlan(N, m=m)
    x1 = torch.tensor(rng.uniform(-0.5, 0.5, (M, 3)), device="cuda")
    x2 = torch.tensor(rng.uniform(-0.5, 0.5, (M, 3)), device="cuda")
    fh = torch.tensor(rng.standard_normal(4096) + 1j * rng.standard_normal(4096), device="cuda")
    fv = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), device="cuda")
    f1 = torch.zeros(M, dtype=torch.complex128, device="cuda")
    f2 = torch.zeros(M, dtype=torch.complex128, device="cuda")
    acc0 = torch.tensor(rng.standard_normal(4096) + 1j * rng.standard_normal(4096), device="cuda")
    acc = acc0.clone()
    s = torch.cuda.Stream()
    L.pnfft_gb300_clear_error()
    lib._check(L.pnfft_gb300_batch_begin(s.cuda_stream or 1), "batch_begin")
    with torch.cuda.stream(s):
        p.trafo_device(x1, fh, lib.COMPUTE_F, f=f1, fixed_nodes=True)
        p.trafo_device(x2, fh, lib.COMPUTE_F, f=f2, fixed_nodes=True)
        p.adj_device(x2, fv, compute_flags=lib.COMPUTE_F | lib.COMPUTE_ACCUMULATED, f_hat=acc, fixed_nodes=True)
    lib._check(L.pnfft_gb300_batch_end(), "batch_end")
    s.synchronize()
    d, n = ctypes.c_int(0), ctypes.c_int(0)
    L.pnfft_gb300_batch_stats(ctypes.byref(d), ctypes.byref(n))
    assert d.value == 3 and n.value == 3  # B of the first call; then B and B^T of the rest
    g1, _, _ = p.trafo_device(x1, fh, lib.COMPUTE_F)
    g2, _, _ = p.trafo_device(x2, fh, lib.COMPUTE_F)
    torch.cuda.synchronize()
    assert torch.equal(f1, g1) and torch.equal(f2, g2)
    xs1, xs2 = x1.cpu().numpy(), x2.cpu().numpy()
    assert _rel(f1.cpu().numpy(), o.trafo(xs1, fh.cpu().numpy())[0]) < 1e-6
    assert _rel(f2.cpu().numpy(), o.trafo(xs2, fh.cpu().numpy())[0]) < 1e-6
    want = acc0.cpu().numpy() + o.adj(xs2, fv.cpu().numpy()).ravel()
    assert _rel(acc.cpu().numpy(), want) < 1e-6


def test_batch_more_calls_than_one_launch_holds(lib, oracle):
    """70 right-hand sides on one node set in one batch: the deferred calls
    of one cutoff go out in launches of at most 64 calls (two here), and every
    result equals its separate call."""
    import ctypes
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    L = lib.load()
    rng = np.random.default_rng(63)
    N, m, M, K = (8, 8, 8), 3, 700, 70
    p = lib.Plan(N, m=m, precision="fp32")
    x = torch.tensor(rng.uniform(-0.5, 0.5, (M, 3)), device="cuda")
    fhs = [torch.tensor(rng.standard_normal(512) + 1j * rng.standard_normal(512), device="cuda") for _ in range(K)]
    outs = [torch.zeros(M, dtype=torch.complex128, device="cuda") for _ in range(K)]
    s = torch.cuda.Stream()
    L.pnfft_gb300_clear_error()
    lib._check(L.pnfft_gb300_batch_begin(s.cuda_stream or 1), "batch_begin")
    with torch.cuda.stream(s):
        for fh, fo in zip(fhs, outs):
            p.trafo_device(x, fh, lib.COMPUTE_F, f=fo, fixed_nodes=True)
    lib._check(L.pnfft_gb300_batch_end(), "batch_end")
    s.synchronize()
    d, n = ctypes.c_int(0), ctypes.c_int(0)
    L.pnfft_gb300_batch_stats(ctypes.byref(d), ctypes.byref(n))
    assert d.value == K and n.value == 2
    o = oracle.OraclePlan(N, m=m)
    xs = x.cpu().numpy()
    for k in (0, 63, 64, 69):
        g, _, _ = p.trafo_device(x, fhs[k], lib.COMPUTE_F)
        torch.cuda.synchronize()
        assert torch.equal(outs[k], g)
        assert _rel(outs[k].cpu().numpy(), o.trafo(xs, fhs[k].cpu().numpy())[0]) < 1e-6
