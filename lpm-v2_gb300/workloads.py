"""Synthetic, seeded workloads of the lpm-v2 direct-sum benchmarks.

Meshes come from the library's PolyMesh2d restatement; initial conditions restate the
reference drivers' vorticity functions:
  GaussianVortexVorticity + SetGaussConst   examples/BVESingleGaussianVortex.f90:335-357
  RossbyHaurwitz54Vorticity                  examples/RossbyHaurwitz54.f90:415-428
  SphericalHarmonicFn (Y_5^4)                tests/SpherePSEConvTest.f90:495-512
  SolidBodyVorticity / SolidBodyVelocity     examples/BVESolidBody.f90:231-243
No dataset or benchmark suite is involved: every input is generated here from a seed.
"""
from __future__ import annotations

import math

import numpy as np

import lpm_gpu as lg

PI = 3.1415926535897932384626433832795027975


def sphere_mesh(seed: int, nest: int, radius: float = 1.0):
    return lg.PolyMesh2d(seed, nest, radius)


def lat_lon_point(lat: float, lon: float, radius: float = 1.0):
    return np.array([radius * math.cos(lon) * math.cos(lat), radius * math.sin(lon) * math.cos(lat),
                     radius * math.sin(lat)])


def gaussian_vortex(mesh, strength: float, shape_sq: float, center, radius: float = 1.0):
    """vortStrength * exp(-shapeParam^2 (a^2 - x.x0)) - GAUSS_CONST, with GAUSS_CONST making
    sum(zeta A) over active particles zero (divided by 4 pi a, SetGaussConst)."""
    dot = mesh.x * center[0] + mesh.y * center[1] + mesh.z * center[2]
    g = strength * np.exp(-shape_sq * (radius * radius - dot))
    act = mesh.active.astype(bool)
    const = np.sum(g[act] * mesh.area[act]) / (4.0 * PI * radius)
    return g - const


def rh54_vorticity(mesh, zonal_wind: float = PI / 7.0, amplitude: float = 1.0, radius: float = 1.0):
    """RossbyHaurwitz54Vorticity: 2 U z/a + 30 A cos(4 lon) P(z/a)/a, P(z) = z (z^2-1)^2."""
    lon = np.arctan2(mesh.y, mesh.x)
    zz = mesh.z / radius
    return 2.0 * zonal_wind * mesh.z / radius + 30.0 * amplitude * np.cos(4.0 * lon) * zz * (zz * zz - 1.0) ** 2 / radius


def y54(x, y, z):
    """SphericalHarmonicFn: 3 sqrt(35) cos(4 lon) sin(lat) (sin(lat)^2 - 1)^2."""
    lat = np.arctan2(z, np.sqrt(x * x + y * y))
    lon = np.arctan2(y, x)
    s = np.sin(lat)
    return 3.0 * math.sqrt(35.0) * np.cos(4.0 * lon) * s * (-1.0 + s * s) ** 2


def y54_surface_gradient(x, y, z):
    """Surface gradient of y54 on the unit sphere: y54 = 3 sqrt(35) z Re((x + i y)^4) is a
    harmonic polynomial of degree 5, so grad_s y54 = grad y54 - 5 y54 p."""
    c = 3.0 * math.sqrt(35.0)
    q = x ** 4 - 6 * x ** 2 * y ** 2 + y ** 4
    y5 = z * q
    gx, gy, gz = z * (4 * x ** 3 - 12 * x * y ** 2), z * (4 * y ** 3 - 12 * x ** 2 * y), q
    return c * (gx - 5 * y5 * x), c * (gy - 5 * y5 * y), c * (gz - 5 * y5 * z)


def colliding_dipoles(x, y, amp: float = 40.0, width_sq: float = 0.04):
    """Two Gaussian dipoles at (+-1, +-0.2) travelling head-on: the dipole at x = -1 has +amp
    above and -amp below (it moves in +x), its mirror image at x = +1 moves in -x."""
    w = np.zeros_like(x)
    for cx, cy, s in ((-1.0, 0.2, 1.0), (-1.0, -0.2, -1.0), (1.0, 0.2, -1.0), (1.0, -0.2, 1.0)):
        w += s * amp * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / width_sq)
    return w


def random_unit_vector(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


# ------------------------------------------------------------------ named configurations
def config_gauss_vortex_icos(nest: int = 4):
    """Single Gaussian vortex, icosahedral mesh: zeta = 4 pi exp(-16 |x - x0|^2), x0 at
    (lat pi/6, lon 0), mean removed; Omega = 2 pi."""
    m = sphere_mesh(lg.ICOS_TRI_SPHERE_SEED, nest)
    x0 = lat_lon_point(PI / 6.0, 0.0)
    zeta = gaussian_vortex(m, 4.0 * PI, 32.0, x0)
    return dict(mesh=m, x=m.x, y=m.y, z=m.z, zeta=zeta, area=m.area, active=m.active, radius=1.0,
                omega=2.0 * PI)


def rh54_velocity(x, y, z, zonal_wind: float = PI / 7.0, amplitude: float = 1.0):
    """Exact velocity of rh54_vorticity on the unit sphere (examples/RossbyHaurwitz54.f90:419-428:
    zeta = 2 w z + 30 K cos(4 lon) z (z^2 - 1)^2).  Its stream function is psi = -w z - K Y with
    Y = z Re((x + i y)^4), a harmonic polynomial of degree 5 (so the surface Laplacian of Y is
    -30 Y), and u = r x grad psi = w (-y, x, 0) - K r x grad Y."""
    gx = z * (4 * x ** 3 - 12 * x * y ** 2)
    gy = z * (4 * y ** 3 - 12 * x ** 2 * y)
    gz = x ** 4 - 6 * x ** 2 * y ** 2 + y ** 4
    return (-zonal_wind * y - amplitude * (y * gz - z * gy), zonal_wind * x - amplitude * (z * gx - x * gz),
            -amplitude * (x * gy - y * gx))


def config_rh54_icos(nest: int = 8, seed: int = 0):
    """RH wave 4 plus a Gaussian vortex (shape 6) at a seeded random centre, mean removed."""
    m = sphere_mesh(lg.ICOS_TRI_SPHERE_SEED, nest)
    rng = np.random.default_rng(seed)
    c = random_unit_vector(rng)
    zeta = rh54_vorticity(m) + gaussian_vortex(m, 4.0 * PI, 36.0, c)
    return dict(mesh=m, x=m.x, y=m.y, z=m.z, zeta=zeta, area=m.area, active=m.active, radius=1.0,
                omega=2.0 * PI)


def config_colliding_dipoles(nest: int = 7, mesh_radius: float = 4.0):
    m = lg.PolyMesh2d(lg.QUAD_RECT_SEED, nest, mesh_radius)
    w = colliding_dipoles(m.x, m.y)
    return dict(mesh=m, x=m.x, y=m.y, omega=w, area=m.area, active=m.active)


def config_beta_plane(nest: int = 7):
    """The beta plane's particle set: the quad refinement on the box [0, 1] x [-1/2, 1/2]
    (src/PolyMesh2d.f90:880-884 maps the seed x -> x/2 + 1/2, y -> y/2), with a Rossby-wave
    vorticity sin(2 pi x) exp(-8 y^2) plus a zonal jet 0.5 tanh(10 y)."""
    m = lg.PolyMesh2d(lg.QUAD_RECT_SEED, nest, 1.0)
    x = 0.5 * m.x + 0.5
    y = 0.5 * m.y
    zeta = np.sin(2.0 * PI * x) * np.exp(-8.0 * y * y) + 0.5 * np.tanh(10.0 * y)
    return dict(x=x, y=y, zeta=zeta, area=0.25 * m.area, active=m.active)


def config_pse_cubed(nest: int = 7, seed: int = 0):
    m = sphere_mesh(lg.CUBED_SPHERE_SEED, nest)
    rng = np.random.default_rng(seed)
    f = y54(m.x, m.y, m.z) + 1e-3 * rng.random(m.n)
    return dict(mesh=m, x=m.x, y=m.y, z=m.z, f=f, area=m.area, active=m.active, radius=1.0,
                eps_k8=m.max_edge_length ** 0.75, eps_gauss=2.0 * m.avg_edge_length)


def config_ensemble(n_instances: int = 64, seed: int = 0, nests=(3, 4, 5, 6)):
    rng = np.random.default_rng(seed)
    meshes = {}
    out = []
    for _ in range(n_instances):
        nest = int(rng.choice(nests))
        if nest not in meshes:
            meshes[nest] = sphere_mesh(lg.ICOS_TRI_SPHERE_SEED, nest)
        m = meshes[nest]
        beta = rng.uniform(2.0, 8.0)
        amp = rng.uniform(2.0 * PI, 6.0 * PI)
        c = random_unit_vector(rng)
        zeta = gaussian_vortex(m, amp, beta * beta, c)
        out.append(dict(x=m.x.copy(), y=m.y.copy(), z=m.z.copy(), rel_vort=zeta, area=m.area.copy(),
                        active=m.active.copy(), radius=1.0, rotation_rate=2.0 * PI, nest=nest))
    return out


def interactions(n_targets: int, n_sources: int, n_active_targets: int | None = None) -> int:
    """N_targets * N_sources minus the excluded self pairs (active targets)."""
    if n_active_targets is None:
        n_active_targets = n_sources
    return n_targets * n_sources - n_active_targets
