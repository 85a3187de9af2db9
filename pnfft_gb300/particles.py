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
  node set, unless the set is fixed (pnfft_gb300_nodes_set_fixed): a node
  set keeps its binning, which serves both directions.

``charge_dipole_host`` runs the whole sequence on host arrays through one C
call, pnfft_gb300_charge_dipole: each node set is copied to the GPU and
binned once for both of its transforms, and f_hat stays on the GPU.

``charges_c2r`` is the real-valued charge-only form: adj(q), then trafo
with the gradient, either analytic or ik-differentiated (PNFFT_DIFF_IK on
the plan).
"""
import ctypes

import numpy as np
import torch

from . import COMPUTE_ACCUMULATED, COMPUTE_F, COMPUTE_GRAD_F, COMPUTE_HESSIAN_F, _check, load
from ._lib import MALLOC_F, MALLOC_GRAD_F, MALLOC_HESSIAN_F, MALLOC_X

__all__ = ["charge_dipole", "charge_dipole_host", "charges_c2r", "HostNodes"]


class HostNodes:
    """A pnfft_nodes object of M nodes owning page-locked host arrays x, f,
    grad_f and hessian_f (PNFFT_MALLOC_*), with numpy views of them."""

    def __init__(self, M):
        L = load()
        self.M = int(M)
        flags = MALLOC_X | MALLOC_F | MALLOC_GRAD_F | MALLOC_HESSIAN_F
        self.handle = L.pnfft_init_nodes(self.M, ctypes.c_uint(flags))
        dp = ctypes.POINTER(ctypes.c_double)

        def view(ptr, n):
            return np.ctypeslib.as_array(ctypes.cast(ptr, dp), (n,)) if self.M else np.zeros(n)

        self.x = view(L.pnfft_get_x(self.handle), 3 * self.M).reshape(-1, 3)
        self.f = view(L.pnfft_get_f(self.handle), 2 * self.M).view(np.complex128)
        self.grad_f = view(L.pnfft_get_grad_f(self.handle), 6 * self.M).view(np.complex128).reshape(-1, 3)
        self.hessian_f = view(L.pnfft_get_hessian_f(self.handle), 12 * self.M).view(np.complex128).reshape(-1, 6)

    def close(self):
        if self.handle:
            load().pnfft_free_nodes(self.handle, ctypes.c_uint(0xF))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Pinned(np.ndarray):
    """A numpy array over page-locked memory from pnfft_alloc_complex, freed with it."""

    def __array_finalize__(self, obj):
        self._owner = getattr(obj, "_owner", None)


class _Block:
    def __init__(self, n):
        self.ptr = load().pnfft_alloc_complex(max(int(n), 1))

    def __del__(self):
        try:
            load().pnfft_free(self.ptr)
        except Exception:
            pass


def _pinned_complex(n):
    blk = _Block(n)
    raw = np.ctypeslib.as_array(ctypes.cast(blk.ptr, ctypes.POINTER(ctypes.c_double)), (2 * max(int(n), 1),))
    arr = raw[:2 * int(n)].view(np.complex128).view(_Pinned)
    arr._owner = blk
    arr[...] = 0
    return arr


def charge_dipole_host(plan, charges, dipoles, compute_flags=0):
    """The sequence of charge_dipole on HostNodes through pnfft_gb300_charge_dipole.

    charges.f holds the charges, dipoles.grad_f the dipole moments.  Returns
    (energy, force, f_hat): energy (Mc + Md,) and force (Mc + Md, 3) complex;
    the node arrays hold phi / grad phi (charges) and grad phi / H (dipoles).
    """
    L = load()
    M = charges.M + dipoles.M
    energy, force = _pinned_complex(M), _pinned_complex(3 * M).reshape(M, 3)
    S = int(np.prod(plan.local_N))
    f_hat = np.zeros(S, np.complex128)
    L.pnfft_set_f_hat(f_hat.ctypes.data, plan._p)
    L.pnfft_gb300_clear_error()
    rc = L.pnfft_gb300_charge_dipole(plan._p, charges.handle, dipoles.handle, ctypes.c_uint(compute_flags),
                                     energy.ctypes.data, force.ctypes.data)
    _check(rc, "pnfft_gb300_charge_dipole")
    return energy, force, f_hat


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
