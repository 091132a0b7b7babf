"""Initial conditions (host-side test-case set-up).

Restatements of the reference's cases in numpy, evaluated on an MPAS mesh
after mesh_init's radius scaling:

* ``mountain_zonal_flow``   - src/test_cases/swm/mountain_zonal_flow_test_mod.F90:25-61
* ``steady_geostrophic_flow`` - src/test_cases/swm/steady_geostrophic_flow_test_mod.F90:20-54
* ``cosine_bell``           - src/test_cases/adv/cosine_bell_rotation_test_mod.F90:22-43
* ``deformation_flow``      - src/test_cases/adv/deformation_flow_test_mod.F90:27-72
* ``jet_zonal_flow``        - src/test_cases/swm/jet_zonal_flow_test_mod.F90:27-84
  (Galewsky, Scott and Polvani 2004: the shipped namelist's case)
* ``rossby_haurwitz_wave``  - src/test_cases/swm/rossby_haurwitz_wave_test_mod.F90:21-63
  (Williamson et al. 1992, case 6)
* ``linearized_rossby_wave`` - src/test_cases/swm/linearized_rossby_wave_test_mod.F90:81-287
  (Shamir and Paldor 2016: an analytic solution at any time t)

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


# ---------------------------------------------------------------------------
# barotropically unstable jet (Galewsky et al. 2004)
# ---------------------------------------------------------------------------
_JET_UMAX = 80.0
_JET_LAT0 = PI / 7.0
_JET_LAT1 = PI / 2.0 - _JET_LAT0
_JET_EN = np.exp(-4.0 / (_JET_LAT1 - _JET_LAT0) ** 2)


def _jet_u(lat):
    """Zonal wind of the jet: u_max/e_n exp(1/((lat-lat0)(lat-lat1))) between lat0 and lat1, else 0."""
    lat = np.asarray(lat, float)
    u = np.zeros_like(lat)
    inside = (lat > _JET_LAT0) & (lat < _JET_LAT1)
    x = lat[inside]
    u[inside] = _JET_UMAX / _JET_EN * np.exp(1.0 / ((x - _JET_LAT0) * (x - _JET_LAT1)))
    return u


def _jet_balance_integral(lat, radius, omega, panels=16, order=16):
    """int_{-pi/2}^{lat} a u (f + tan(phi) u / a) dphi for each lat, by composite
    Gauss-Legendre quadrature over [lat0, min(lat, lat1)] (the integrand is zero
    outside the jet): about 1e-12 relative.  The reference uses QUADPACK's qags
    with epsrel 1e-3 (jet_zonal_flow_test_mod.F90:50), whose result differs from
    this by at most its error estimate."""
    lat = np.asarray(lat, float)
    top = np.clip(lat, _JET_LAT0, _JET_LAT1)
    x, w = np.polynomial.legendre.leggauss(order)
    out = np.zeros_like(lat)
    width = (top - _JET_LAT0) / panels
    for p in range(panels):
        lo = _JET_LAT0 + p * width
        phi = lo[:, None] + 0.5 * width[:, None] * (x[None, :] + 1.0)
        u = _jet_u(phi)
        f = 2.0 * omega * np.sin(phi)
        out += 0.5 * width * np.sum(w[None, :] * radius * u * (f + np.tan(phi) / radius * u), axis=1)
    return out


def jet_zonal_flow(mesh, radius=REF_RADIUS, g=REF_G, omega=REF_OMEGA):
    """Galewsky jet: the balanced zonal jet with its 120-m Gaussian depth bump at
    45 degrees north (jet_zonal_flow_test_mod.F90:27-61); no topography.  u on
    an edge is cos(angleEdge) |u(latEdge)|."""
    ghd, lat2, alpha, beta = g * 120.0, PI / 4.0, 1.0 / 3.0, 1.0 / 15.0
    u = np.cos(mesh.angleEdge) * np.abs(_jet_u(mesh.latEdge))
    gd = g * 1.0e4 - _jet_balance_integral(mesh.latCell, radius, omega)
    lon = np.where(mesh.lonCell > PI, mesh.lonCell - 2.0 * PI, mesh.lonCell)
    gd = gd + ghd * np.cos(mesh.latCell) * np.exp(-(lon / alpha) ** 2) * np.exp(-((lat2 - mesh.latCell) / beta) ** 2)
    return gd, u, np.zeros(mesh.nCells)


# ---------------------------------------------------------------------------
# Rossby-Haurwitz wave of wavenumber 4 (Williamson et al. 1992, case 6)
# ---------------------------------------------------------------------------
# The reference writes w and K as single-precision literals (7.848e-6 without a
# kind), so their values are the FP32 roundings promoted to FP64.
RH_W = float(np.float32(7.848e-6))
RH_K = RH_W
RH_R = 4.0
RH_H0 = 8000.0


def rossby_haurwitz_wave(mesh, radius=REF_RADIUS, g=REF_G, omega=REF_OMEGA):
    """Velocity from the vertex streamfunction differenced over dvEdge, depth
    from the balance relation (rossby_haurwitz_wave_test_mod.F90:21-63)."""
    w, K, R = RH_W, RH_K, RH_R
    a2 = radius * radius
    latv, lonv = mesh.latVertex, mesh.lonVertex
    psi = -a2 * w * np.sin(latv) + a2 * K * np.cos(latv) ** R * np.sin(latv) * np.cos(R * lonv)
    u = _uv_from_psi(mesh, psi, radius)
    c = np.cos(mesh.latCell)
    aa = 0.5 * w * (2.0 * omega + w) * c ** 2 + 0.25 * K ** 2 * c ** (2.0 * R) * (
        (R + 1.0) * c ** 2 + 2.0 * R ** 2 - R - 2.0 - 2.0 * R ** 2 * c ** (-2.0))
    bb = (2.0 * (omega + w) * K / ((R + 1.0) * (R + 2.0))) * c ** R * ((R ** 2 + 2.0 * R + 2.0) - ((R + 1.0) * c) ** 2)
    cc = 0.25 * K ** 2 * c ** (2.0 * R) * ((R + 1.0) * c ** 2 - R - 2.0)
    lon = mesh.lonCell
    gd = g * RH_H0 + a2 * aa + a2 * bb * np.cos(R * lon) + a2 * cc * np.cos(2.0 * R * lon)
    return gd, u, np.zeros(mesh.nCells)


def rossby_haurwitz_angular_speed(omega=REF_OMEGA):
    """Angular phase speed of the wave pattern in the non-divergent limit,
    (R (3 + R) w - 2 Omega) / ((1 + R)(2 + R)) rad/s (Haurwitz 1940)."""
    R, w = RH_R, RH_W
    return (R * (3.0 + R) * w - 2.0 * omega) / ((1.0 + R) * (2.0 + R))


# ---------------------------------------------------------------------------
# linear Rossby wave, analytic (Shamir and Paldor 2016), mode n = 5, k = 10
# ---------------------------------------------------------------------------
LRW_H0 = 5.0e3
LRW_N = 5
LRW_K = 10
LRW_SIGMA = 0.5 + (0.25 + LRW_K ** 2) ** 0.5


def lrw_phase_speed(radius=REF_RADIUS, g=REF_G, omega=REF_OMEGA):
    """Phase speed (rad/s) of the Rossby mode: the smallest-magnitude root of
    the cubic dispersion relation, negative (westward)."""
    k, n, s = LRW_K, LRW_N, LRW_SIGMA
    gh = g * LRW_H0
    en = gh / radius ** 2 * (n + s) ** 2
    d0 = 3.0 * k ** 2 * en
    d4 = -54.0 * k ** 4 * gh * omega / radius ** 2
    roots = []
    for j in (1, 2, 3):
        dj = complex(d4 ** 2 - 4.0 * d0 ** 3) ** 0.5
        dj = (0.5 * (d4 + dj)) ** (1.0 / 3.0)
        dj = dj * np.exp(2.0j * PI * j / 3.0)
        roots.append((-1.0 / 3.0 / k ** 2 * (dj + d0 / dj)).real)
    return -min(abs(r) for r in roots)


def _lrw_amplitudes(lat, radius, g, omega):
    """Latitude amplitudes (u~, v~, h~) of the Rossby mode."""
    s, k = LRW_SIGMA, LRW_K
    a3 = s * (s + 1) * (s + 2)
    a4 = a3 * (s + 3)
    a5 = a4 * (s + 4)
    amp = 1.0e-8
    sl, cl = np.sin(lat), np.cos(lat)
    c5 = (4.0 * a5 * sl ** 4 - 20.0 * a4 * sl ** 2 + 15.0 * a3) * sl / 15.0
    c5p = (4.0 * a5 * sl ** 4 - 12.0 * a4 * sl ** 2 + 3.0 * a3) * cl / 3.0
    psi = amp * cl ** s * c5
    dpsi = amp * cl ** s * (-s * np.tan(lat) * c5 + c5p)
    C = lrw_phase_speed(radius, g, omega)
    o2 = 2.0 * omega
    kp = (g * LRW_H0 + radius ** 2 * C ** 2 * cl ** 2) / (C * cl)
    km = (g * LRW_H0 - radius ** 2 * C ** 2 * cl ** 2) / (C * cl)
    vt = (o2 * np.abs(km) / cl ** 2) ** 0.5 * psi
    ht = (o2 * np.abs(km) * radius ** 2 * LRW_H0 ** 2) ** 0.5 / km * (dpsi + np.tan(lat) * (0.5 * kp / km - o2 / C) * psi)
    ut = (o2 * sl / C) * vt + (g / radius / cl / C) * ht
    return ut, k * vt, ht


def linearized_rossby_wave(mesh, t=0.0, radius=REF_RADIUS, g=REF_G, omega=REF_OMEGA):
    """The analytic Rossby-mode solution at time t (s): depth H0 + h~ cos(k lon -
    k C t) on cells, and the normal component of (u, v) on edges, u = u~ cos(k
    lon - k C t), v = v~ sin(k lon - k C t).  The reference forms the normal
    component as cos(theta - angleEdge) |(u, v)| with theta the direction of
    (u, v) (linearized_rossby_wave_test_mod.F90:81-103); here it is
    u cos(angleEdge) + v sin(angleEdge), the same number up to rounding."""
    k, C = LRW_K, lrw_phase_speed(radius, g, omega)
    _, _, ht = _lrw_amplitudes(mesh.latCell, radius, g, omega)
    h = ht * np.cos(k * mesh.lonCell - k * C * t) + LRW_H0
    ut, vt, _ = _lrw_amplitudes(mesh.latEdge, radius, g, omega)
    ph = k * mesh.lonEdge - k * C * t
    ue, ve = ut * np.cos(ph), vt * np.cos(ph - 0.5 * PI)
    u = ue * np.cos(mesh.angleEdge) + ve * np.sin(mesh.angleEdge)
    return h * g, u, np.zeros(mesh.nCells)


# the shallow-water cases by their namelist name (test_cases_mod.F90:17-34), plus
# the benchmark's seeded case; each returns (gd, u, ghs)
SWM_CASES = ("jet_bumps", "mountain_zonal_flow", "steady_geostrophic_flow", "rossby_haurwitz_wave",
             "linearized_rossby_wave", "jet_zonal_flow")


def by_name(name: str, mesh, seed: int = 0):
    """Initial (gd, u, ghs) of the named shallow-water case."""
    if name == "jet_bumps":
        return jet_bumps(mesh, seed=seed)
    if name not in SWM_CASES:
        raise ValueError(f"unknown case {name!r}; one of {', '.join(SWM_CASES)}")
    return globals()[name](mesh)
