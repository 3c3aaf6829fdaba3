"""Golden fixture for the analytic-solution tests (solCx and solKz of the reference's performance
tests): the analytic velocity and pressure at the 2 x 2 Gauss points of every element of 16^2,
32^2 and 64^2 unit-square meshes (FP32), from the reference's own analytic plugin sources
(Underworld/SysTest/AnalyticPlugins/Velic_solCx/solCx.c and Velic_solKz/solKz.c, compiled here with
gcc into oracle/_ref/), and the convergence rates the reference's expected results state.

- solCx (Underworld/SysTest/PerformanceTests/testVelicSolCx.xml): etaA = 100 for x < 0.5, etaB = 1,
  n = 2; expected rates (PerformanceTests/expected/Underworld_Velic_solCx-analysis.cvg-convergence-
  rates.dat): velocity 1.99 / 1.99, pressure 1.00.
- solKz (PerformanceTests/testVelicSolKz.xml): sigma = 1, km = pi, n = 1, B = 1 (viscosity
  exp(2 y)); expected rates (Underworld_Velic_solKz-analysis.cvg-convergence-rates.dat): velocity
  2.00 / 2.00, pressure 1.00.
- solA (testVelicSolA.xml): isoviscous (Z = 1), buoyancy Ra T with T = sin(3.5 pi y) cos(pi x)
  (VelicTemperatureIC), solA's sigma = 1, n = 1, km = 3.5 pi; solB (testVelicSolB.xml): isoviscous,
  T = sinh(2 y) cos(pi x) (VelicTemperatureIC_SolB), sigma = 1, n = 1, km = 2; solS
  (testVelicSolS.xml): isoviscous, no buoyancy, top lid v_x = sin(pi x) (Velocity_SinusoidalLid),
  bottom no-slip, side walls v_x = 0, n = 1, eta = 1.  Their expected rates are read from
  Underworld_Velic_sol{A,B,S}-analysis.cvg-convergence-rates.dat (velocity x, y, pressure).

Usage: python tests/golden/make_velic_golden.py <path of the Underworld 1.x source tree>
"""
import ctypes as C
import math
import os
import subprocess
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit(__doc__)
REF = sys.argv[1]
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT_DIR = os.path.join(REPO, "oracle", "_ref")
os.makedirs(OUT_DIR, exist_ok=True)
D = C.POINTER(C.c_double)


def build(name):
    src = os.path.join(REF, "Underworld", "SysTest", "AnalyticPlugins", f"Velic_{name}", f"{name}.c")
    lib = os.path.join(OUT_DIR, f"lib{name}.so")
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-DNOSHARED", src, "-o", lib, "-lm"])
    return C.CDLL(lib)


cx = build("solCx")
cx._Velic_solCx.argtypes = [D, C.c_double, C.c_double, C.c_double, C.c_int, D, D, D, D]
kz = build("solKz")
kz._Velic_solKz.argtypes = [D, C.c_double, C.c_double, C.c_int, C.c_double, D, D, D, D]
sa = build("solA")
sa._Velic_solA.argtypes = [D, C.c_double, C.c_double, C.c_int, C.c_double, D, D, D, D]
sb = build("solB")
sb._Velic_solB.argtypes = [D, C.c_double, C.c_double, C.c_int, C.c_double, D, D, D, D]
ss = build("solS")
ss._Velic_solS.argtypes = [D, C.c_int, C.c_double, D, D, D, D]


def expected_rates(name):
    """velocity x, velocity y and pressure rates of the reference's convergence-rate file"""
    path = os.path.join(REF, "Underworld", "SysTest", "PerformanceTests", "expected",
                        f"Underworld_Velic_{name}-analysis.cvg-convergence-rates.dat")
    line = [l for l in open(path) if l.startswith("cvg. rate")][0]
    return [float(v) for v in line.split()[2:5]]


def call(f, x, y, *params):
    pos = (C.c_double * 2)(x, y)
    vel = (C.c_double * 2)()
    p = C.c_double()
    st = (C.c_double * 3)()
    sr = (C.c_double * 3)()
    f(pos, *params, vel, C.byref(p), st, sr)
    return vel[0], vel[1], p.value


CASES = {
    "cx": (lambda x, y: call(cx._Velic_solCx, x, y, 100.0, 1.0, 0.5, 2), [1.99, 1.99, 1.00]),
    "kz": (lambda x, y: call(kz._Velic_solKz, x, y, 1.0, math.pi, 1, 1.0), [2.00, 2.00, 1.00]),
    "a": (lambda x, y: call(sa._Velic_solA, x, y, 1.0, 1.0, 1, 3.5 * math.pi), expected_rates("solA")),
    "b": (lambda x, y: call(sb._Velic_solB, x, y, 1.0, 1.0, 1, 2.0), expected_rates("solB")),
    "s": (lambda x, y: call(ss._Velic_solS, x, y, 1, 1.0), expected_rates("solS")),
}
g = (1.0 - 1.0 / np.sqrt(3.0)) / 2.0
LOC = [(g, g), (1 - g, g), (g, 1 - g), (1 - g, 1 - g)]
out = {}
for case, (fn, rates) in CASES.items():
    out[f"{case}_expected_rates"] = np.array(rates)
    for n in (16, 32, 64):
        ug = np.zeros((n * n * 4, 2))
        pg = np.zeros(n * n * 4)
        for j in range(n):
            for i in range(n):
                for q, (a, b) in enumerate(LOC):
                    vx, vy, pp = fn((i + a) / n, (j + b) / n)
                    ug[(j * n + i) * 4 + q] = (vx, vy)
                    pg[(j * n + i) * 4 + q] = pp
        out[f"{case}_ug_{n}"] = ug.astype(np.float32)
        out[f"{case}_pg_{n}"] = pg.astype(np.float32)
np.savez_compressed(os.path.join(HERE, "velic_golden.npz"), **out)
print("wrote", os.path.join(HERE, "velic_golden.npz"))
