"""Golden fixture for the solCx analytic-solution test: the analytic velocity and pressure at the
2 x 2 Gauss points of every element of 16^2, 32^2 and 64^2 unit-square meshes (FP32), from the reference's
own analytic plugin source (Underworld/SysTest/AnalyticPlugins/Velic_solCx/solCx.c, compiled here
with gcc into oracle/_ref/), for the parameters of Underworld/SysTest/PerformanceTests/
testVelicSolCx.xml (etaA = 100 for x < 0.5, etaB = 1, n = 2), and the reference's expected
convergence rates of that test (PerformanceTests/expected/
Underworld_Velic_solCx-analysis.cvg-convergence-rates.dat: velocity 1.99 / 1.99, pressure 1.00).

Usage: python tests/golden/make_solcx_golden.py <path of the Underworld 1.x source tree>
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit(__doc__)
REF = sys.argv[1]
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(REF, "Underworld", "SysTest", "AnalyticPlugins", "Velic_solCx", "solCx.c")
OUT_DIR = os.path.join(REPO, "oracle", "_ref")
LIB = os.path.join(OUT_DIR, "libsolcx.so")
os.makedirs(OUT_DIR, exist_ok=True)
subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-DNOSHARED", SRC, "-o", LIB, "-lm"])
lib = C.CDLL(LIB)
D = C.POINTER(C.c_double)
lib._Velic_solCx.argtypes = [D, C.c_double, C.c_double, C.c_double, C.c_int, D, D, D, D]
lib._Velic_solCx.restype = None
ETA_A, ETA_B, XC, N = 100.0, 1.0, 0.5, 2


def solcx(x, y):
    pos = (C.c_double * 2)(x, y)
    vel = (C.c_double * 2)()
    p = C.c_double()
    st = (C.c_double * 3)()
    sr = (C.c_double * 3)()
    lib._Velic_solCx(pos, ETA_A, ETA_B, XC, N, vel, C.byref(p), st, sr)
    return vel[0], vel[1], p.value


out = {"params": np.array([ETA_A, ETA_B, XC, N]),
       "expected_rates": np.array([1.99, 1.99, 1.00])}
for n in (16, 32, 64):
    # 2 x 2 Gauss points of every element (local +-1/sqrt(3)), element-major, for the L2 norms the
    # reference's FieldTest integrates (PICellerator/... gaussSwarm)
    g = (1.0 - 1.0 / np.sqrt(3.0)) / 2.0
    loc = [(g, g), (1 - g, g), (g, 1 - g), (1 - g, 1 - g)]
    ug = np.zeros((n * n * 4, 2))
    pg = np.zeros(n * n * 4)
    for j in range(n):
        for i in range(n):
            for q, (a, b) in enumerate(loc):
                vx, vy, pp = solcx((i + a) / n, (j + b) / n)
                ug[(j * n + i) * 4 + q] = (vx, vy)
                pg[(j * n + i) * 4 + q] = pp
    out[f"ug_{n}"] = ug.astype(np.float32)
    out[f"pg_{n}"] = pg.astype(np.float32)
np.savez_compressed(os.path.join(HERE, "solcx_golden.npz"), **out)
print("wrote", os.path.join(HERE, "solcx_golden.npz"))
