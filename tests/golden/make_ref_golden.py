"""Writes tests/golden/ref_golden.npz: outputs of the reference PNFFT itself
(oracle/_ref/libpnfft_ref.so, its own C code built against single-process
stand-ins, oracle/build_ref.py) on small seeded inputs, one entry per case.
Run from the repository root where the reference tree is present:
    python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import pnfft_oracle as O  # noqa: E402
from oracle import reference as R  # noqa: E402

CASES = {
    # name: (N, n, m, flags, cflags)
    "kb_m3": ((8, 8, 8), (16, 16, 16), 3, 0, 7),
    "kb_m6_sigma": ((8, 6, 10), (12, 12, 16), 6, 0, 3),
    "gaussian_interlaced": ((8, 8, 8), (16, 16, 16), 4, O.WINDOW_GAUSSIAN | O.INTERLACED, 3),
    "bspline_ik": ((8, 8, 8), (16, 16, 16), 3, O.WINDOW_BSPLINE | O.DIFF_IK, 3),
    "sinc_power": ((8, 8, 8), (16, 16, 16), 3, O.WINDOW_SINC_POWER, 7),
    "bessel_i0_cub": ((8, 8, 8), (16, 16, 16), 4, O.WINDOW_BESSEL_I0 | O.PRE_CUB_PSI, 3),
    "gaussian_t_quad": ((8, 8, 8), (16, 16, 16), 3, O.WINDOW_GAUSSIAN_T | O.PRE_QUAD_PSI, 1),
}


def main():
    out = {}
    for i, (name, (N, n, m, flags, cflags)) in enumerate(CASES.items()):
        rng = np.random.default_rng(1000 + i)
        M = 200
        S = int(np.prod(N))
        x = rng.uniform(-0.5, 0.5, (M, 3))
        fh = rng.standard_normal(S) + 1j * rng.standard_normal(S)
        f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
        g = rng.standard_normal((M, 3)) + 1j * rng.standard_normal((M, 3))
        r = R.RefPlan(N, n, m=m, flags=flags)
        tf, tg, th = r.trafo(x, fh, cflags)
        adj = r.adj(x, f, g, O.COMPUTE_F | O.COMPUTE_GRAD_F)
        d = {"N": np.array(N), "n": np.array(n), "m": np.array(m), "flags": np.array(flags),
             "cflags": np.array(cflags), "x": x, "f_hat": fh, "f": f, "grad": g, "trafo_f": tf, "adj": adj}
        if cflags & O.COMPUTE_GRAD_F:
            d["trafo_grad"] = tg
        if cflags & O.COMPUTE_HESSIAN_F:
            d["trafo_hess"] = th
        for k, v in d.items():
            out[name + "/" + k] = v
        r.close()
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
