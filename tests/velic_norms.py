"""L2 error norms of a Q1-P0 solution against the analytic solutions of the reference's performance
tests (solCx, solKz: the norms its FieldTest integrates with a 2 x 2 Gauss swarm), from the fixture
tests/golden/velic_golden.npz, and the convergence rates of the three norms."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "velic_golden.npz")
G = (1.0 - 1.0 / np.sqrt(3.0)) / 2.0
LOC = [(G, G), (1 - G, G), (G, 1 - G), (1 - G, 1 - G)]


def golden():
    return np.load(GOLDEN)


def errors(case, n, u, p, g):
    """u: nodal velocity (nn, 2) (node = i + (n + 1) j), p: element pressures (n^2); -> L2 errors of
    vx, vy and p (pressure compared after removing each field's integrated mean)."""
    ug = g[f"{case}_ug_{n}"].astype(np.float64).reshape(n * n, 4, 2)
    pg = g[f"{case}_pg_{n}"].astype(np.float64).reshape(n * n, 4)
    e = np.arange(n * n)
    i, j = e % n, e // n
    n00, n10 = i + (n + 1) * j, i + 1 + (n + 1) * j
    n01, n11 = n00 + n + 1, n10 + n + 1
    w = 1.0 / (4.0 * n * n)   # 2 x 2 Gauss weights x detJ of an element of side 1/n
    ev = np.zeros(2)
    for q, (a, b) in enumerate(LOC):
        uh = (1 - a) * (1 - b) * u[n00] + a * (1 - b) * u[n10] + (1 - a) * b * u[n01] + a * b * u[n11]
        ev += w * np.sum((uh - ug[:, q, :]) ** 2, axis=0)
    ph = p - np.mean(p)
    pa = pg - np.sum(w * pg)   # integrated mean of the unit square
    ep = np.sqrt(np.sum(w * (ph[:, None] - pa) ** 2))
    return np.array([np.sqrt(ev[0]), np.sqrt(ev[1]), ep])


def rates(errs, ns):
    h = 1.0 / np.asarray(ns, dtype=np.float64)
    return np.array([np.polyfit(np.log(h), np.log(errs[:, k]), 1)[0] for k in range(errs.shape[1])])
