"""Seeded synthetic inputs for the Stokes workloads this library is measured on.

Each generator returns a dict with the mesh, the material points (x, y, z, material index,
optional per-point viscosity/density), the material table, the boundary mask and the force
settings.  No public dataset is involved: the inputs follow the workload descriptions
(layouts, shapes, value ranges) with fixed seeds.

Workloads:
  rt2d     2D Rayleigh-Taylor, 64x64, 20 points/element, Park-Miller layout stream
           (StgDomain/Swarm/src/Random.c, RandomParticleLayout.c), BelowCosinePlane interface
  spheres  3D 64^3, 27 points/element on a jittered 3x3x3 grid, 50 seeded spheres
  grf      3D 128^3, 30 uniform points/element, log10(viscosity) a Gaussian random field
  layers   3D 96^3, 40 points/element, Arrhenius + Drucker-Prager + limiter (nonlinear)
  solcx    2D analytic-solution case of the reference's performance tests (viscosity jump)
  solkz    2D analytic-solution case of the reference's performance tests (exponential viscosity)
"""
from __future__ import annotations

import numpy as np

from . import uwgpu as U

PM_A = 16807
PM_M = 2147483647


def park_miller_stream(seed: int, count: int) -> np.ndarray:
    """States 1..count of the Park-Miller generator seeded as Swarm_Random_Seed(seed)."""
    s0 = (seed ^ 123459876) % PM_M
    block = 4096
    first = np.empty(block, np.int64)
    x = s0
    for i in range(block):
        x = (PM_A * x) % PM_M
        first[i] = x
    if count <= block:
        return first[:count].astype(np.float64)
    aB = pow(PM_A, block, PM_M)
    out = np.empty(((count + block - 1) // block) * block, np.int64)
    cur = first
    for b in range(0, out.shape[0], block):
        out[b:b + block] = cur
        cur = (cur * aB) % PM_M
    return out[:count].astype(np.float64)


def _element_origin(nel, h, e):
    dim = len(nel)
    ex = e % nel[0]
    ey = (e // nel[0]) % nel[1]
    out = [ex * h[0], ey * h[1]]
    if dim == 3:
        out.append((e // (nel[0] * nel[1])) * h[2])
    return out


def _node_coord(i, n, mn=0.0, mx=1.0):
    i = np.asarray(i)
    v = mn + (i / n) * (mx - mn)
    return np.where(i <= 0, mn, np.where(i >= n, mx, v))


def rt2d(nel=(64, 64), ppc=20, seed=13):
    """2D Rayleigh-Taylor: dense layer (rho=1, eta=1) over a light layer (rho=0, eta=0.01)
    below y = 0.2 + 0.02 cos(pi x); free-slip walls; gravity (0, -1)."""
    nx, ny = nel
    E = nx * ny
    r = park_miller_stream(seed, E * ppc * 3).reshape(E, ppc, 3)
    ex = np.arange(E) % nx
    ey = np.arange(E) // nx
    x0, x1 = _node_coord(ex, nx), _node_coord(ex + 1, nx)
    y0, y1 = _node_coord(ey, ny), _node_coord(ey + 1, ny)
    x = (x1 - x0)[:, None] * r[:, :, 0] / float(PM_M) + x0[:, None]
    y = (y1 - y0)[:, None] * r[:, :, 1] / float(PM_M) + y0[:, None]
    x = x.reshape(-1)
    y = y.reshape(-1)
    below = y < 0.2 + 0.02 * np.cos(2 * np.pi * x / 2.0)
    mat = np.where(below, 1, 0).astype(np.int32)
    mats = [U.make_material([(U.LAW_MATERIAL_VISCOSITY, [1.0])], density=1.0),
            U.make_material([(U.LAW_MATERIAL_VISCOSITY, [0.01])], density=0.0)]
    return dict(name="rt2d", dim=2, nel=tuple(nel), x=x, y=y, z=None, material=mat, eta=None, rho=None,
                materials=mats, fixed=U.free_slip_mask(2, nel), gravity=1.0, vert_axis=1, seed=seed,
                mg_levels=4)


def solcx(n=64, ppc=20, seed=13, eta_a=100.0, eta_b=1.0, xc=0.5, ky=2.0):
    """2D solCx (Underworld/SysTest/PerformanceTests/testVelicSolCx.xml): viscosity eta_a left of
    x = xc and eta_b right of it, a nodal temperature T = sin(ky pi y) cos(pi x) (VelicTemperatureIC,
    StgFEM/plugins/StandardConditionFunctions/StandardConditionFunctions.c:1298-1338) driving the
    buoyancy as rho = -T (density 1e-12 with expansivity 1e12 about T = 0, so rho = 1e-12 - T), g = 1;
    free-slip walls; ppc points per element on the Park-Miller layout of the reference's test."""
    E = n * n
    r = park_miller_stream(seed, E * ppc * 3).reshape(E, ppc, 3)
    ex = np.arange(E) % n
    ey = np.arange(E) // n
    x0, x1 = _node_coord(ex, n), _node_coord(ex + 1, n)
    y0, y1 = _node_coord(ey, n), _node_coord(ey + 1, n)
    x = ((x1 - x0)[:, None] * r[:, :, 0] / float(PM_M) + x0[:, None]).reshape(-1)
    y = ((y1 - y0)[:, None] * r[:, :, 1] / float(PM_M) + y0[:, None]).reshape(-1)
    mat = np.where(x < xc, 0, 1).astype(np.int32)
    mats = [U.make_material([(U.LAW_MATERIAL_VISCOSITY, [eta_a])], density=1e-12, alpha=1e12, ref_temp=0.0),
            U.make_material([(U.LAW_MATERIAL_VISCOSITY, [eta_b])], density=1e-12, alpha=1e12, ref_temp=0.0)]
    k = np.arange((n + 1) ** 2)
    xn, yn = _node_coord(k % (n + 1), n), _node_coord(k // (n + 1), n)
    temp = np.sin(ky * np.pi * yn) * np.cos(np.pi * xn)
    return dict(name="solcx", dim=2, nel=(n, n), x=x, y=y, z=None, material=mat, eta=None, rho=None,
                materials=mats, fixed=U.free_slip_mask(2, (n, n)), gravity=1.0, vert_axis=1, seed=seed,
                temperature=temp, mg_levels=3)


def solkz(n=64, ppc=20, seed=13, twice_b=2.0, km_waves=1.0):
    """2D solKz (Underworld/SysTest/PerformanceTests/testVelicSolKz.xml): viscosity exp(twice_b y)
    (DepthDependentViscosity along y, eta0 1, reference point 0), temperature
    T = sin(km_waves pi y) cos(pi x) driving the buoyancy as rho = -T, g = 1; free-slip walls; ppc
    points per element on the Park-Miller layout."""
    w = solcx(n, ppc, seed, ky=km_waves)
    law = [(U.LAW_DEPTH_DEPENDENT, [1.0, twice_b, 0.0, 1.0])]
    w["materials"] = [U.make_material(law, density=1e-12, alpha=1e12, ref_temp=0.0)]
    w["material"] = np.zeros_like(w["material"])
    w["name"] = "solkz"
    return w


def spheres(nel=(64, 64, 64), nspheres=50, seed=2024, jitter=0.15, shuffle=True):
    """3D: 27 points per element on a 3x3x3 grid at cell fractions 1/6, 1/2, 5/6, each jittered by
    U(-jitter, jitter) of the cell width; background eta 1 / rho 0; spheres radius U(0.05, 0.15),
    eta 10^U(-2, 3), rho U(0, 1); a later sphere overwrites an earlier one."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = nel
    E = nx * ny * nz
    fr = np.array([1.0 / 6.0, 0.5, 5.0 / 6.0])
    gi, gj, gk = np.meshgrid(fr, fr, fr, indexing="ij")
    base = np.stack([gi.reshape(-1), gj.reshape(-1), gk.reshape(-1)], axis=1)  # 27 x 3 (x,y,z)
    e = np.arange(E)
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    pts = []
    for d, (ei, n) in enumerate(((ex, nx), (ey, ny), (ez, nz))):
        c0, c1 = _node_coord(ei, n), _node_coord(ei + 1, n)
        frac = base[None, :, d] + rng.uniform(-jitter, jitter, size=(E, 27))
        pts.append((c0[:, None] + (c1 - c0)[:, None] * frac).reshape(-1))
    x, y, z = pts
    centres = rng.uniform(0.0, 1.0, size=(nspheres, 3))
    radii = rng.uniform(0.05, 0.15, size=nspheres)
    etas = 10.0 ** rng.uniform(-2.0, 3.0, size=nspheres)
    rhos = rng.uniform(0.0, 1.0, size=nspheres)
    mat = np.zeros(x.shape[0], np.int32)
    for s in range(nspheres):
        inside = (x - centres[s, 0]) ** 2 + (y - centres[s, 1]) ** 2 + (z - centres[s, 2]) ** 2 <= radii[s] ** 2
        mat[inside] = s + 1
    mats = [U.make_material([(U.LAW_MATERIAL_VISCOSITY, [1.0])], density=0.0)]
    for s in range(nspheres):
        mats.append(U.make_material([(U.LAW_MATERIAL_VISCOSITY, [etas[s]])], density=rhos[s]))
    if shuffle:
        # material-point storage after advection is not element ordered
        order = rng.permutation(x.shape[0])
        x, y, z, mat = x[order], y[order], z[order], mat[order]
    return dict(name="spheres", dim=3, nel=tuple(nel), x=x, y=y, z=z, material=mat, eta=None, rho=None,
                materials=mats, fixed=U.free_slip_mask(3, nel), gravity=1.0, vert_axis=2, seed=seed,
                mg_levels=4)


def gaussian_random_field(n=256, corr=0.1, seed=7):
    """Periodic GRF on an n^3 grid with squared-exponential covariance (spectral synthesis)."""
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n, d=1.0 / n) * 2 * np.pi
    kx, ky, kz = np.meshgrid(k, k, k[: n // 2 + 1], indexing="ij", sparse=True)
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    spec = np.exp(-0.25 * k2 * corr * corr)  # sqrt of the SE power spectrum (up to a constant)
    noise = rng.standard_normal((n, n, n))
    f = np.fft.irfftn(np.fft.rfftn(noise) * spec, s=(n, n, n), axes=(0, 1, 2))
    f -= f.mean()
    f /= np.abs(f).max()
    return f


def _trilinear(field, x, y, z):
    n = field.shape[0]
    gx, gy, gz = x * n, y * n, z * n
    i0 = np.floor(gx).astype(np.int64)
    j0 = np.floor(gy).astype(np.int64)
    k0 = np.floor(gz).astype(np.int64)
    fx, fy, fz = gx - i0, gy - j0, gz - k0
    out = np.zeros_like(x)
    for di in (0, 1):
        wx = fx if di else 1 - fx
        for dj in (0, 1):
            wy = fy if dj else 1 - fy
            for dk in (0, 1):
                wz = fz if dk else 1 - fz
                out += wx * wy * wz * field[(i0 + di) % n, (j0 + dj) % n, (k0 + dk) % n]
    return out


def grf(nel=(128, 128, 128), ppc=30, seed=11, grid=256, corr=0.1, shuffle=True):
    """3D: uniform random points; log10(eta) = GRF scaled to [-3, 3] (1e6 contrast);
    rho = 0.5 * g + 0.5 with g the field normalised to [-1, 1]."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = nel
    E = nx * ny * nz
    e = np.repeat(np.arange(E), ppc)
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    pts = []
    for ei, n in ((ex, nx), (ey, ny), (ez, nz)):
        c0, c1 = _node_coord(ei, n), _node_coord(ei + 1, n)
        pts.append(c0 + (c1 - c0) * rng.uniform(0.0, 1.0, size=E * ppc))
    x, y, z = pts
    g = gaussian_random_field(grid, corr, seed + 1)
    gp = _trilinear(g, x, y, z)
    gp = gp / np.abs(gp).max()
    eta = 10.0 ** (3.0 * gp)
    rho = 0.5 * gp + 0.5
    mats = [U.make_material([(U.LAW_PARTICLE_VISCOSITY, [])], density=0.0)]
    mat = np.zeros(x.shape[0], np.int32)
    if shuffle:
        order = rng.permutation(x.shape[0])
        x, y, z, eta, rho = x[order], y[order], z[order], eta[order], rho[order]
    return dict(name="grf", dim=3, nel=tuple(nel), x=x, y=y, z=z, material=mat, eta=eta, rho=rho,
                materials=mats, fixed=U.free_slip_mask(3, nel), gravity=1.0, vert_axis=2, seed=seed,
                mg_levels=5)


def layers(nel=(96, 96, 96), ppc=40, seed=5, nbumps=20, cohesion_scale=1.0):
    """3D nonlinear: 5 horizontal layers (seeded thicknesses), T = 1 - z + sum of 20 Gaussian
    bumps (amplitude 0.1, width 0.05); per layer Arrhenius eta = exp(E/(T+0.1) - E/1.1) with
    E ~ U(5, 15), Drucker-Prager with C ~ U(0.1, 1), mu = 0.6, then a [1e-3, 1e3] limiter."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = nel
    E = nx * ny * nz
    e = np.repeat(np.arange(E), ppc)
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    pts = []
    for ei, n in ((ex, nx), (ey, ny), (ez, nz)):
        c0, c1 = _node_coord(ei, n), _node_coord(ei + 1, n)
        pts.append(c0 + (c1 - c0) * rng.uniform(0.0, 1.0, size=E * ppc))
    x, y, z = pts
    th = rng.uniform(0.5, 1.5, size=5)
    bounds = np.concatenate([[0.0], np.cumsum(th) / th.sum()])
    layer = np.clip(np.searchsorted(bounds, z, side="right") - 1, 0, 4).astype(np.int32)
    mats = []
    for _ in range(5):
        Ea = rng.uniform(5.0, 15.0)
        coh = rng.uniform(0.1, 1.0) * cohesion_scale
        rho = rng.uniform(0.0, 1.0)   # layer density (seeded; drives the flow)
        mats.append(U.make_material([(U.LAW_ARRHENIUS, [np.exp(-Ea / 1.1), Ea, 0.0, 0.1]),
                                     (U.LAW_DRUCKER_PRAGER, [coh, 0.6, 0.0, 1e-3]),
                                     (U.LAW_VISCOSITY_LIMITER, [1e3, 1e-3])], density=rho))
    centres = rng.uniform(0.0, 1.0, size=(nbumps, 3))
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    idx = np.arange(nn)
    X = _node_coord(idx % (nx + 1), nx)
    Y = _node_coord((idx // (nx + 1)) % (ny + 1), ny)
    Z = _node_coord(idx // ((nx + 1) * (ny + 1)), nz)
    T = 1.0 - Z
    for b in range(nbumps):
        T = T + 0.1 * np.exp(-((X - centres[b, 0]) ** 2 + (Y - centres[b, 1]) ** 2 + (Z - centres[b, 2]) ** 2) / (2 * 0.05 ** 2))
    return dict(name="layers", dim=3, nel=tuple(nel), x=x, y=y, z=z, material=layer, eta=None, rho=None,
                materials=mats, fixed=U.free_slip_mask(3, nel), gravity=1.0, vert_axis=2, seed=seed,
                temperature=T, mg_levels=4)


def driven_walls(dim, nel, kind="lid"):
    """Non-zero Dirichlet conditions of two driven models, as (fixed mask, values), node-major
    (node * dim + component):
      lid        free-slip walls, and on the top wall (y = 1 in 2D, z = 1 in 3D) the x velocity
                 fixed to 4 x (1 - x) (zero at the corners, so no net flux through any wall)
      extension  x walls pulled apart (u_x = -0.5 at x = 0, +0.5 at x = 1), the other side walls
                 and the bottom free-slip, the top open"""
    nx, ny = nel[0] + 1, nel[1] + 1
    nz = nel[2] + 1 if dim == 3 else 1
    idx = np.arange(nx * ny * nz)
    i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    X = _node_coord(i, nel[0])
    fixed = np.zeros((idx.size, dim), np.uint8)
    val = np.zeros((idx.size, dim))
    top = (j == ny - 1) if dim == 2 else (k == nz - 1)
    if kind == "lid":
        fixed[:] = U.free_slip_mask(dim, nel).reshape(-1, dim)
        fixed[top, 0] = 1
        val[top, 0] = 4.0 * X[top] * (1.0 - X[top])
    elif kind == "extension":
        fixed[(i == 0) | (i == nx - 1), 0] = 1
        val[i == 0, 0] = -0.5
        val[i == nx - 1, 0] = 0.5
        if dim == 2:
            fixed[j == 0, 1] = 1
        else:
            fixed[(j == 0) | (j == ny - 1), 1] = 1
            fixed[k == 0, 2] = 1
    else:
        raise ValueError(kind)
    return fixed.reshape(-1), val.reshape(-1)


def setup_context(ctx: U.Context, w: dict):
    """Load a workload into a device context (mesh, BCs, materials, fields, points)."""
    dim = w["dim"]
    ctx.mesh_q1(dim, w["nel"])
    ctx.bc_set(w["fixed"], w.get("bcval"))
    ctx.materials_set(w["materials"])
    ctx.fields_set(w.get("temperature"), w.get("gravity", 0.0), w.get("vert_axis", dim - 1))
    ctx.particles_upload(w["x"], w["y"], w["z"], w["material"], w.get("eta"), w.get("rho"))
