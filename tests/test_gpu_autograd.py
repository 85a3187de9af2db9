"""torch.autograd.Function over the C ABI (pnfft_gb300.autograd.trafo):
gradients against FP64 central finite differences of the same transform and
against the oracle's PNFFT_COMPUTE_GRAD_F."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _loss(P, torch, plan, fh, x, y):
    from pnfft_gb300.autograd import trafo
    f = trafo(fh, x, plan)
    return (torch.abs(f - y) ** 2).sum()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-7), ("fp32", 2e-4)])
def test_gradients_vs_central_differences(lib, prec, tol):
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device")
    P = lib
    N, M = (8, 8, 8), 64
    rng = np.random.default_rng(21)
    plan = P.Plan(N, m=6, precision=prec)
    ref = P.Plan(N, m=6, precision="fp64")
    x0 = rng.uniform(-0.45, 0.45, (M, 3))
    fh0 = rng.standard_normal(512) + 1j * rng.standard_normal(512)
    y = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), device="cuda")
    x = torch.tensor(x0, device="cuda", requires_grad=True)
    fh = torch.tensor(fh0, device="cuda", requires_grad=True)
    L = _loss(P, torch, plan, fh, x, y)
    L.backward()
    gx = x.grad.cpu().numpy()
    gfh = fh.grad.cpu().numpy()

    def L64(xn, fhn):
        with torch.no_grad():
            return _loss(P, torch, ref, torch.tensor(fhn, device="cuda"), torch.tensor(xn, device="cuda"), y).item()

    h = 1e-6
    scale_x = np.abs(gx).max()
    for j, t in [(0, 0), (5, 1), (17, 2), (40, 0), (63, 2)]:
        xp, xm = x0.copy(), x0.copy()
        xp[j, t] += h
        xm[j, t] -= h
        fd = (L64(xp, fh0) - L64(xm, fh0)) / (2 * h)
        assert abs(fd - gx[j, t]) <= tol * scale_x, (j, t, fd, gx[j, t])
    scale_f = np.abs(gfh).max()
    for k in [0, 7, 100, 255, 511]:
        fp, fm = fh0.copy(), fh0.copy()
        fp[k] += h
        fm[k] -= h
        d_re = (L64(x0, fp) - L64(x0, fm)) / (2 * h)
        fp, fm = fh0.copy(), fh0.copy()
        fp[k] += 1j * h
        fm[k] -= 1j * h
        d_im = (L64(x0, fp) - L64(x0, fm)) / (2 * h)
        assert abs(complex(d_re, d_im) - gfh[k]) <= tol * scale_f, (k, d_re, d_im, gfh[k])


def test_grad_x_matches_compute_grad_f(lib, oracle):
    torch = pytest.importorskip("torch")
    P = lib
    N, M = (16, 16, 16), 300
    rng = np.random.default_rng(22)
    x0 = rng.uniform(-0.5, 0.5, (M, 3))
    fh0 = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
    plan = P.Plan(N, m=6, precision="fp64")
    x = torch.tensor(x0, device="cuda", requires_grad=True)
    fh = torch.tensor(fh0, device="cuda")
    from pnfft_gb300.autograd import trafo
    f = trafo(fh, x, plan)
    g = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), device="cuda")
    f.backward(g)
    o = oracle.OraclePlan(N, m=6)
    _, grad_f, _ = o.trafo(x0, fh0, oracle.COMPUTE_GRAD_F)
    want = (np.conj(g.cpu().numpy())[:, None] * grad_f).real
    got = x.grad.cpu().numpy()
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12


def test_autograd_full_size_vs_fp64_central_differences(lib):
    # the autograd workload: N=64^3, n=128^3, M=2^20, FP32-mixed plan, float32
    # coordinates; FP64 central differences (h=1e-6) on 256 coordinates and
    # 32 f_hat entries.  Differences are formed per node (the loss of 2^20
    # terms would cancel): x_jt changes only f_j, and the loss is quadratic
    # in f_hat with trafo(f_hat + h e_k) = f + h trafo(e_k).
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device")
    from pnfft_gb300.autograd import trafo
    rng = np.random.default_rng(23)
    N, M, h = (64, 64, 64), 2 ** 20, 1e-6
    S = 64 ** 3
    plan = lib.Plan(N, m=6, precision="fp32")
    ref = lib.Plan(N, m=6, precision="fp64")
    x = torch.tensor(rng.uniform(-0.5, 0.5, (M, 3)), dtype=torch.float32, device="cuda", requires_grad=True)
    fh = torch.tensor(rng.standard_normal(S) + 1j * rng.standard_normal(S), device="cuda", requires_grad=True)
    y = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), device="cuda")
    L = (torch.abs(trafo(fh, x, plan) - y) ** 2).sum()
    L.backward()
    x64 = x.detach().to(torch.float64)
    fh64 = fh.detach()
    with torch.no_grad():
        f64, _, _ = ref.trafo_device(x64, fh64)
        r = f64 - y
        # coordinates
        js = torch.tensor(rng.choice(M, 256, replace=False), device="cuda")
        ts = torch.tensor(rng.integers(0, 3, 256), device="cuda")
        xs = x64[js].clone()
        xp, xm = xs.clone(), xs.clone()
        xp[torch.arange(256), ts] += h
        xm[torch.arange(256), ts] -= h
        fpm, _, _ = ref.trafo_device(torch.cat([xp, xm]).contiguous(), fh64)
        fd = (torch.abs(fpm[:256] - y[js]) ** 2 - torch.abs(fpm[256:] - y[js]) ** 2) / (2 * h)
        ad = x.grad[js, ts].to(torch.float64)
        err_x = (torch.linalg.vector_norm(ad - fd) / torch.linalg.vector_norm(fd)).item()
        # f_hat entries
        ks = rng.choice(S, 32, replace=False)
        fd_fh, ad_fh = [], []
        for k in ks:
            e = torch.zeros(S, dtype=torch.complex128, device="cuda")
            e[int(k)] = 1.0
            gk, _, _ = ref.trafo_device(x64, e)
            d_re = (torch.abs(r + h * gk) ** 2 - torch.abs(r - h * gk) ** 2).sum() / (2 * h)
            d_im = (torch.abs(r + 1j * h * gk) ** 2 - torch.abs(r - 1j * h * gk) ** 2).sum() / (2 * h)
            fd_fh.append(complex(d_re.item(), d_im.item()))
            ad_fh.append(complex(fh.grad[int(k)].item()))
        fd_fh, ad_fh = np.array(fd_fh), np.array(ad_fh)
        err_f = np.linalg.norm(ad_fh - fd_fh) / np.linalg.norm(fd_fh)
    assert err_x < 1e-6, err_x
    assert err_f < 1e-6, err_f
