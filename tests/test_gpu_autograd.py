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
