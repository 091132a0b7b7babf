"""Initial conditions (host-side test-case set-up).

Restatements of the reference's cases in numpy, evaluated on an MPAS mesh
after mesh_init's radius scaling:

* ``mountain_zonal_flow``   - src/test_cases/swm/mountain_zonal_flow_test_mod.F90:25-61
* ``steady_geostrophic_flow`` - src/test_cases/swm/steady_geostrophic_flow_test_mod.F90:20-54
* ``cosine_bell``           - src/test_cases/adv/cosine_bell_rotation_test_mod.F90:22-43
* ``deformation_flow``      - src/test_cases/adv/deformation_flow_test_mod.F90:27-72

plus the seeded ``jet_bumps`` case of the project's benchmark (no reference
counterpart): a balanced zonal jet u = u0 cos(lat) built like
mountain_zonal_flow (vertex streamfunction differenced over dvEdge, so the
discrete flow is non-divergent), a seeded spherical-harmonic depth
perturbation over degrees 4-16 at 1% of h0, and 8 Gaussian mountains; and
``smooth_tracers``: seeded fields in [0, 1] made of degree <= 8 harmonics.
"""
from __future__ import annotations

import numpy as np

from .gpu import REF_G, REF_OMEGA, REF_RADIUS

PI = 4.0 * np.arctan(1.0)


def _uv_from_psi(mesh, psi_vertex, radius):
    v1 = mesh.verticesOnEdge[:, 0] - 1
    v2 = mesh.verticesOnEdge[:, 1] - 1
    dv = mesh.dvEdge * radius
    return -(psi_vertex[v2] - psi_vertex[v1]) / dv


def mountain_zonal_flow(mesh, radius=REF_RADIUS, g=REF_G, omega=REF_OMEGA):
    alpha, u0, gd0 = 0.0, 20.0, 5960.0 * g
    lon0, lat0, ghs0, R = PI * 1.5, PI / 6.0, 2000.0 * g, PI / 9.0
    dlon = np.abs(mesh.lonCell - lon0)
    dlon = np.minimum(dlon, 2 * PI - dlon)
    d = np.minimum(R, np.sqrt(dlon ** 2 + (mesh.latCell - lat0) ** 2))
    ghs = ghs0 * (1.0 - d / R)
    ca, sa = np.cos(alpha), np.sin(alpha)
    psi = -radius * u0 * (np.sin(mesh.latVertex) * ca - np.cos(mesh.lonVertex) * np.cos(mesh.latVertex) * sa)
    u = _uv_from_psi(mesh, psi, radius)
    gd = gd0 - (radius * omega * u0 + 0.5 * u0 ** 2) * (
        -np.cos(mesh.lonCell) * np.cos(mesh.latCell) * sa + np.sin(mesh.latCell) * ca) ** 2 - ghs
    return gd, u, ghs


def steady_geostrophic_flow(mesh, radius=REF_RADIUS, g=REF_G, omega=REF_OMEGA):
    alpha = 0.0
    u0 = 2 * PI * radius / (12 * 86400)
    gd0 = 2.94e4
    psi = -radius * u0 * (np.sin(mesh.latVertex) * np.cos(alpha)
                          - np.cos(mesh.lonVertex) * np.cos(mesh.latVertex) * np.sin(alpha))
    u = _uv_from_psi(mesh, psi, radius)
    gd = gd0 - (radius * omega * u0 + 0.5 * u0 ** 2.0) * (
        -np.cos(mesh.lonCell) * np.cos(mesh.latCell) * np.sin(alpha) + np.sin(mesh.latCell) * np.cos(alpha)) ** 2.0
    return gd, u, np.zeros(mesh.nCells)


def _legendre_all(lmax, x):
    """Fully normalised associated Legendre functions P[l][m](x), x = sin(lat)."""
    c = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    P = {}
    pmm = np.ones_like(x)
    for m in range(lmax + 1):
        if m == 1:
            pmm = np.sqrt(3.0) * c
        elif m > 1:
            pmm = pmm * c * np.sqrt((2.0 * m + 1.0) / (2.0 * m))
        P[(m, m)] = pmm
        if m + 1 <= lmax:
            P[(m + 1, m)] = np.sqrt(2.0 * m + 3.0) * x * pmm
        for l in range(m + 2, lmax + 1):
            a = np.sqrt((2.0 * l - 1.0) * (2.0 * l + 1.0) / ((l - m) * (l + m)))
            b = np.sqrt((2.0 * l + 1.0) * (l + m - 1.0) * (l - m - 1.0) / ((l - m) * (l + m) * (2.0 * l - 3.0)))
            P[(l, m)] = a * x * P[(l - 1, m)] - b * P[(l - 2, m)]
    return P


_BASIS_CACHE: list = []


def _basis(lat, lon, lmax):
    """Legendre table and cos/sin(m lon) of one set of points (cached per array pair)."""
    for la, lo, lm, val in _BASIS_CACHE:
        if la is lat and lo is lon and lm >= lmax:
            return val
    P = _legendre_all(lmax, np.sin(lat))
    cm = [np.cos(m * lon) for m in range(lmax + 1)]
    sm = [np.sin(m * lon) for m in range(lmax + 1)]
    val = (P, cm, sm)
    _BASIS_CACHE.append((lat, lon, lmax, val))
    del _BASIS_CACHE[:-4]
    return val


def harmonic_field(lat, lon, lmin, lmax, rng):
    """Sum of real spherical harmonics of degrees lmin..lmax with N(0,1) coefficients."""
    P, cm, sm = _basis(lat, lon, lmax)
    f = np.zeros_like(lat)
    for l in range(lmin, lmax + 1):
        for m in range(0, l + 1):
            a, b = rng.standard_normal(2)
            if m == 0:
                f += a * P[(l, 0)]
            else:
                f += P[(l, m)] * (a * cm[m] + b * sm[m])
    return f


def _great_circle(lat1, lon1, lat2, lon2):
    s = np.sin(lat1) * np.sin(lat2) + np.cos(lat1) * np.cos(lat2) * np.cos(lon1 - lon2)
    return np.arccos(np.clip(s, -1.0, 1.0))


def jet_bumps(mesh, seed: int, radius=REF_RADIUS, g=REF_G, omega=REF_OMEGA, h0=5000.0):
    """Seeded balanced jet + SH perturbation (degrees 4-16, 1% of h0) + 8 Gaussian mountains."""
    rng = np.random.default_rng(seed)
    u0 = rng.uniform(10.0, 40.0)
    # 8 Gaussian bumps: centres uniform on the sphere, heights 500-2000 m, widths 500-1500 km
    clat = np.arcsin(rng.uniform(-1.0, 1.0, 8))
    clon = rng.uniform(0.0, 2 * PI, 8)
    hb = rng.uniform(500.0, 2000.0, 8)
    wb = rng.uniform(500e3, 1500e3, 8)
    hs = np.zeros(mesh.nCells)
    for k in range(8):
        d = radius * _great_circle(mesh.latCell, mesh.lonCell, clat[k], clon[k])
        hs += hb[k] * np.exp(-(d / wb[k]) ** 2)
    ghs = g * hs
    psi = -radius * u0 * np.sin(mesh.latVertex)
    u = _uv_from_psi(mesh, psi, radius)
    pert = harmonic_field(mesh.latCell, mesh.lonCell, 4, 16, np.random.default_rng(seed + 7919))
    pert *= 0.01 * h0 / np.max(np.abs(pert))
    gd = g * h0 - (radius * omega * u0 + 0.5 * u0 ** 2) * np.sin(mesh.latCell) ** 2 - ghs + g * pert
    return gd, u, ghs


def smooth_tracers(mesh, n: int, seed: int, lmax: int = 8):
    """n tracer mixing ratios in [0, 1] from harmonics of degree <= lmax."""
    out = np.empty((n, mesh.nCells))
    for k in range(n):
        f = harmonic_field(mesh.latCell, mesh.lonCell, 0, lmax, np.random.default_rng(seed * 1000 + k))
        out[k] = (f - f.min()) / (f.max() - f.min())
    return out


def cosine_bell(mesh, radius=REF_RADIUS):
    """Tracer of cosine_bell_rotation_test_mod.F90:29-40 (the wind is set by the model)."""
    h0, lon0, lat0, R0 = 1000.0, 1.5 * PI, 0.0, radius / 3.0
    r = radius * np.arccos(np.sin(lat0) * np.sin(mesh.latCell) + np.cos(lat0) * np.cos(mesh.latCell)
                           * np.cos(mesh.lonCell - lon0))
    return np.where(r < R0, 0.5 * R0 * (1.0 + np.cos(PI * r / R0)), 0.0)


def deformation_flow(mesh, subcase: str = "gaussian_hills", radius=REF_RADIUS, g=REF_G):
    """Tracer of deformation_flow_test_mod.F90:27-72 (case4 winds are set by the model)."""
    lon1, lat1, lon2, lat2 = PI * 5.0 / 6.0, 0.0, PI * 7.0 / 6.0, 0.0
    x1, y1, z1 = np.cos(lat1) * np.cos(lon1), np.cos(lat1) * np.sin(lon1), np.sin(lat1)
    x2, y2, z2 = np.cos(lat2) * np.cos(lon2), np.cos(lat2) * np.sin(lon2), np.sin(lat2)
    if subcase == "gaussian_hills":
        xc, yc, zc = mesh.xCell * radius, mesh.yCell * radius, mesh.zCell * radius
        d1 = ((x1 - xc) ** 2 + (y1 - yc) ** 2 + (z1 - zc) ** 2) / radius ** 2
        d2 = ((x2 - xc) ** 2 + (y2 - yc) ** 2 + (z2 - zc) ** 2) / radius ** 2
        return 0.95 * (np.exp(-5.0 * d1) + np.exp(-5.0 * d2))
    if subcase == "slotted_cylinders":
        r, b, c = 0.5 * radius, 0.1 * g, 1.0 * g
        lat, lon = mesh.latCell, mesh.lonCell
        r1 = radius * _great_circle(lat1, lon1, lat, lon)
        r2 = radius * _great_circle(lat2, lon2, lat, lon)
        q = np.full(mesh.nCells, b)
        m1 = (r1 <= r) & (np.abs(lon - lon1) >= r / 6.0 / radius)
        m2 = (r2 <= r) & (np.abs(lon - lon2) >= r / 6.0 / radius)
        m3 = (r1 <= r) & (np.abs(lon - lon1) < r / 6.0 / radius) & (lat - lat1 < -5.0 / 12.0 * r / radius)
        m4 = (r2 <= r) & (np.abs(lon - lon2) < r / 6.0 / radius) & (lat - lat2 > 5.0 / 12.0 * r / radius)
        q[m1 | m2 | m3 | m4] = c
        return q
    raise ValueError(subcase)
