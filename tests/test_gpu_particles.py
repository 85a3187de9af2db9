"""Particle-mesh caller patterns (pnfft_gb300.particles) against the oracle
running the same sequence: the charge/dipole sequence of the reference's
tests/check_charge_dipole.c:151-233 (c2c) and the clustered real-valued
charge system of the particle workload (c2r; Gaussian and B-spline windows,
analytic and ik gradients)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def clustered_nodes(rng, M, frac=0.2, ncl=64, sigma=0.01):
    """80% uniform in [-0.5, 0.5)^3, 20% from isotropic Gaussian clusters
    (centres uniform), wrapped periodically into [-0.5, 0.5)."""
    mc = int(frac * M)
    x = rng.uniform(-0.5, 0.5, (M, 3))
    centres = rng.uniform(-0.5, 0.5, (ncl, 3))
    pick = rng.integers(0, ncl, mc)
    x[:mc] = centres[pick] + sigma * rng.standard_normal((mc, 3))
    return np.mod(x + 0.5, 1.0) - 0.5


def neutral_charges(rng, M):
    q = np.where(np.arange(M) % 2 == 0, 1.0, -1.0)
    rng.shuffle(q)
    return q


def test_charge_dipole_sequence(lib, oracle):
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    from pnfft_gb300.particles import charge_dipole
    rng = np.random.default_rng(61)
    N, m = (16, 16, 16), 5
    xc, xd = rng.uniform(-0.5, 0.5, (300, 3)), rng.uniform(-0.5, 0.5, (200, 3))
    q = rng.standard_normal(300) + 0j
    mu = rng.standard_normal((200, 3)) + 0j
    o = oracle.OraclePlan(N, m=m)
    fh = o.adj(xc, q)
    fh = o.adj(xd, None, mu, oracle.COMPUTE_GRAD_F) + fh
    phi, gphi, _ = o.trafo(xc, fh, oracle.COMPUTE_F | oracle.COMPUTE_GRAD_F)
    _, gd, hd = o.trafo(xd, fh, oracle.COMPUTE_GRAD_F | oracle.COMPUTE_HESSIAN_F)
    want = [q * phi, gphi * q[:, None], (gd * mu).sum(1),
            np.stack([hd[:, 0] * mu[:, 0] + hd[:, 1] * mu[:, 1] + hd[:, 2] * mu[:, 2],
                      hd[:, 1] * mu[:, 0] + hd[:, 3] * mu[:, 1] + hd[:, 4] * mu[:, 2],
                      hd[:, 2] * mu[:, 0] + hd[:, 4] * mu[:, 1] + hd[:, 5] * mu[:, 2]], 1), fh]
    T = lambda a: torch.tensor(a, device="cuda")  # noqa: E731
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-6)):
        p = lib.Plan(N, m=m, precision=prec)
        got = charge_dipole(p, T(xc), T(q), T(xd), T(mu))
        for g, w in zip(got, want):
            assert _rel(g.cpu().numpy(), w) < tol, prec


@pytest.mark.parametrize("win", ["gaussian", "bspline"])
@pytest.mark.parametrize("ik", [False, True])
def test_clustered_c2r_charges(lib, oracle, win, ik):
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    from pnfft_gb300.particles import charges_c2r
    rng = np.random.default_rng(62)
    N, m, M = (32, 32, 32), 5, 20000
    x = clustered_nodes(rng, M)
    q = neutral_charges(rng, M)
    flags = {"gaussian": lib.WINDOW_GAUSSIAN, "bspline": lib.WINDOW_BSPLINE}[win] | (lib.DIFF_IK if ik else 0)
    o = oracle.OraclePlan(N, m=m, flags=flags, c2r=True)
    fh = o.adj(x, q)
    phi, gphi, _ = o.trafo(x, fh, oracle.COMPUTE_F | oracle.COMPUTE_GRAD_F)
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-6)):
        p = lib.Plan(N, m=m, flags=flags, c2r=True, precision=prec)
        g_fh, g_phi, g_gphi = charges_c2r(p, torch.tensor(x, device="cuda"), torch.tensor(q, device="cuda"))
        assert _rel(g_fh.cpu().numpy(), fh) < tol, prec
        assert _rel(g_phi.cpu().numpy(), phi) < tol, prec
        assert _rel(g_gphi.cpu().numpy(), gphi) < tol, prec


def test_charge_dipole_one_c_call(lib, oracle):
    # pnfft_gb300_charge_dipole: the four transforms and the energies and
    # forces in one C call on host node arrays; each node set is binned once
    # (by its adjoint), so the trafos record no sort time
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    from pnfft_gb300.particles import HostNodes, charge_dipole_host
    rng = np.random.default_rng(63)
    N, m, Mc, Md = (16, 16, 16), 5, 3000, 1000
    xc, xd = rng.uniform(-0.5, 0.5, (Mc, 3)), rng.uniform(-0.5, 0.5, (Md, 3))
    q = rng.standard_normal(Mc) + 0j
    mu = rng.standard_normal((Md, 3)) + 0j
    o = oracle.OraclePlan(N, m=m)
    fh = o.adj(xc, q)
    fh = o.adj(xd, None, mu, oracle.COMPUTE_GRAD_F) + fh
    phi, gphi, _ = o.trafo(xc, fh, oracle.COMPUTE_F | oracle.COMPUTE_GRAD_F)
    _, gd, hd = o.trafo(xd, fh, oracle.COMPUTE_GRAD_F | oracle.COMPUTE_HESSIAN_F)
    w_energy = np.concatenate([q * phi, (gd * mu).sum(1)])
    w_force = np.concatenate([gphi * q[:, None],
                              np.stack([hd[:, 0] * mu[:, 0] + hd[:, 1] * mu[:, 1] + hd[:, 2] * mu[:, 2],
                                        hd[:, 1] * mu[:, 0] + hd[:, 3] * mu[:, 1] + hd[:, 4] * mu[:, 2],
                                        hd[:, 2] * mu[:, 0] + hd[:, 4] * mu[:, 1] + hd[:, 5] * mu[:, 2]], 1)])
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-6)):
        p = lib.Plan(N, m=m, precision=prec)
        ch, di = HostNodes(Mc), HostNodes(Md)
        for _ in range(2):  # a second call with the same arrays gives the same result
            ch.x[:] = xc
            ch.f[:] = q
            di.x[:] = xd
            di.grad_f[:] = mu
            energy, force, f_hat = charge_dipole_host(p, ch, di)
            assert _rel(f_hat, fh) < tol, prec
            assert _rel(energy, w_energy) < tol, prec
            assert _rel(force, w_force) < tol, prec
            assert _rel(ch.f, phi) < tol and _rel(ch.grad_f, gphi) < tol, prec
            assert _rel(di.grad_f, gd) < tol and _rel(di.hessian_f, hd) < tol, prec
            assert p.stage_ms(False)[lib.TIMER_SORT_NODES] == 0.0  # the dipoles' trafo did not bin
            assert p.stage_ms(True)[lib.TIMER_SORT_NODES] > 0.0   # their adjoint did
        ch.close()
        di.close()
        p.close()
