"""Particle-mesh caller patterns of PNFFT on device arrays.

The reference's particle test (tests/check_charge_dipole.c:151-233) drives
the transforms in a fixed sequence:
1. f_hat = adj(charges, COMPUTE_F);
2. f_hat += adj(dipoles, COMPUTE_GRAD_F);
3. trafo(charges, COMPUTE_F | COMPUTE_GRAD_F): the potential and field at
   each charge;
4. trafo(dipoles, COMPUTE_GRAD_F | COMPUTE_HESSIAN_F): the field and field
   gradient at each dipole.
It then forms the per-particle energies and forces:
- charges: q phi and q grad phi;
- dipoles: mu . grad phi and H mu.

Here the same sequence runs on torch CUDA tensors through the C ABI:
- the second adjoint accumulates into f_hat with COMPUTE_ACCUMULATED, where
  the reference copies f_hat into a buffer and adds it back;
- one plan serves both node sets, as in the reference; each call bins its
  node set (the binning cache of a plan holds one node set per direction).

``charges_c2r`` is the real-valued charge-only form: adj(q), then trafo
with the gradient, either analytic or ik-differentiated (PNFFT_DIFF_IK on
the plan).
"""
import torch

from . import COMPUTE_ACCUMULATED, COMPUTE_F, COMPUTE_GRAD_F, COMPUTE_HESSIAN_F

__all__ = ["charge_dipole", "charges_c2r"]


def charge_dipole(plan, xc, q, xd, mu):
    """c2c charges q (Mc) at xc (Mc,3) and dipoles mu (Md,3) at xd (Md,3).

    Returns (energy_c, force_c, energy_d, force_d, f_hat) with energy_c = q*phi,
    force_c = q*grad phi (Mc,3), energy_d = mu.grad phi, force_d = H mu (Md,3).
    """
    S = 1
    for v in plan.local_N:
        S *= v
    f_hat = torch.empty(S, dtype=torch.complex128, device=q.device)
    plan.adj_device(xc, q, compute_flags=COMPUTE_F, f_hat=f_hat)
    plan.adj_device(xd, None, mu, compute_flags=COMPUTE_GRAD_F | COMPUTE_ACCUMULATED, f_hat=f_hat)
    phi, gphi, _ = plan.trafo_device(xc, f_hat, COMPUTE_F | COMPUTE_GRAD_F)
    _, gd, hd = plan.trafo_device(xd, f_hat, COMPUTE_GRAD_F | COMPUTE_HESSIAN_F)
    energy_c = q * phi
    force_c = gphi * q[:, None]
    energy_d = (gd * mu).sum(1)
    h = hd  # xx, xy, xz, yy, yz, zz
    force_d = torch.stack([h[:, 0] * mu[:, 0] + h[:, 1] * mu[:, 1] + h[:, 2] * mu[:, 2],
                           h[:, 1] * mu[:, 0] + h[:, 3] * mu[:, 1] + h[:, 4] * mu[:, 2],
                           h[:, 2] * mu[:, 0] + h[:, 4] * mu[:, 1] + h[:, 5] * mu[:, 2]], 1)
    return energy_c, force_c, energy_d, force_d, f_hat


def charges_c2r(plan, x, q):
    """Real charges q (M,) at x (M,3) on a c2r plan.

    Returns (f_hat, phi, grad_phi): the charge spectrum, and the potential
    and its gradient at the charges.
    """
    f_hat = plan.adj_device(x, q, compute_flags=COMPUTE_F)
    phi, gphi, _ = plan.trafo_device(x, f_hat, COMPUTE_F | COMPUTE_GRAD_F)
    return f_hat, phi, gphi
