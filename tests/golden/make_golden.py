"""Regenerates the golden vectors of tests/golden/ (committed outputs).

special.json   -- scipy values of I0 and Re erf(a+iy), the functions the
                  reference takes from GSL (kernel/bessel_i0.c:375) and libcerf
                  (kernel/matrix_D.c:43).
rand_inputs.json -- the node and sample generators of the reference
                  (api/api-adv.c:35-86, api/api-basic.c:681-691) evaluated here
                  with the C library's own srand/rand through ctypes, i.e.
                  independently of the oracle's C code.
Run:  python tests/golden/make_golden.py
"""
import ctypes
import json
import os

import numpy as np
import scipy.special

HERE = os.path.dirname(os.path.abspath(__file__))


def special():
    i0 = [[float(x), float(scipy.special.i0(x))] for x in (0.0, 0.5, 3.0, 11.3, 28.27, 47.1)]
    erf = []
    for a in (1.2, 3.7599, 5.0):
        for y in (0.25, 1.7, 2.6):
            erf.append([a, y, float(scipy.special.erf(complex(a, y)).real)])
    return {"i0": i0, "re_erf": erf}


def rand_inputs():
    libc = ctypes.CDLL(None)
    libc.rand.restype = ctypes.c_int
    RAND_MAX = 2147483647

    def lt1():
        while True:
            t = libc.rand() / RAND_MAX
            if t < 1.0:
                return t

    libc.srand(0)
    x = []
    for _ in range(8):
        for _t in range(3):
            while True:
                v = (0.5 - (-0.5)) * lt1() + (-0.5)
                if -0.5 <= v < 0.5:
                    break
            x.append(v)
    libc.srand(1)
    f = []
    for _ in range(4):
        f.append(100.0 * libc.rand() / RAND_MAX)
        f.append(100.0 * libc.rand() / RAND_MAX)
    return {"x_srand0": x, "f_srand1": f}


if __name__ == "__main__":
    with open(os.path.join(HERE, "special.json"), "w") as fh:
        json.dump(special(), fh, indent=1)
    with open(os.path.join(HERE, "rand_inputs.json"), "w") as fh:
        json.dump(rand_inputs(), fh, indent=1)
    print("written")
