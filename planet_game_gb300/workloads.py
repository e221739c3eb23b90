"""Seeded synthetic inputs of the heat-transport workloads (numpy, host side).

All workloads are synthetic: there is no dataset. Every generator takes a seed and
uses numpy's PCG64 generator, so inputs are reproducible bit for bit on any host.

* ``step_inputs``: one implicit heat-transport sub-step - T0 = 288 K - 40 K sin^2(lat)
  + N(0, 0.5 K), S = 0.7 Q - (203.3 + 2.09 (T0 - 273.15)) W/m^2 with Q the sub-step-mean
  insolation of sub-step 0, C = 4e7 J/m^2/K, edge diffusivity 1e6 m^2/s (conductance
  C kappa), dt = one twelfth of the reference planet's orbital period.
* ``harmonic_field``: sums of real spherical harmonics l <= lmax with N(0, 1)
  coefficients, with their analytic surface gradient (east, north), Laplacian and exact
  edge-normal fluxes of the gradient at edge midpoints.
* ``column_profiles``: N equal-mass layers over p_s = 1000 hPa (layer bottoms
  1000, 900, ... hPa for N = 10), a 6.5 K/km lapse rate from the surface temperature,
  humidity 0.8 q_sat, seeded cloud fraction U(0, 1) as cloud water f W_c / m.
* ``planet_mix`` / ``poisson_trace``: the batched and served workloads.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ORBITAL_PERIOD_S = 31_556_925.216          # the reference planet's orbital period
SUBSTEP_S = ORBITAL_PERIOD_S / 12.0        # one climate sub-step (1/12 year)
HEAT_CAPACITY = 4.0e7                      # J/m^2/K
DIFFUSIVITY = 1.0e6                        # m^2/s
EARTH_RADIUS = 6.371e6
EARTH_GRAVITY = 6.67430e-11 * 5.9722e24 / (6.371e6 * 6.371e6)
STEFAN_BOLTZMANN = 5.670374419e-8

# Earth-like column constants: tau_d, kappa_v (atmosphere.hpp:120-121), W_c, r_e, g,
# kappa_l (atmosphere.hpp:79-82), p0, gravity, sigma.
EARTH_COLUMN = dict(dry_optical_depth=1.1298583872, vapour_absorption_m2_kg=0.005649291936,
                    in_cloud_water_path_kg_m2=0.05, effective_radius_m=18e-6, cloud_asymmetry=0.85,
                    cloud_longwave_absorption_m2_kg=130.0, reference_pressure_Pa=101_325.0,
                    gravity_m_s2=EARTH_GRAVITY, stefan_boltzmann=STEFAN_BOLTZMANN)


def latitude(center: np.ndarray) -> np.ndarray:
    return np.arcsin(np.clip(center[:, 2], -1.0, 1.0))


def initial_temperature(center: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    lat = latitude(center)
    return 288.0 - 40.0 * np.sin(lat) ** 2 + rng.normal(0.0, 0.5, len(center))


def source_term(insolation: np.ndarray, t0: np.ndarray) -> np.ndarray:
    return 0.7 * insolation.astype(np.float64) - (203.3 + 2.09 * (t0 - 273.15))


@dataclass
class StepInputs:
    t0: np.ndarray
    source: np.ndarray
    heat_capacity: float
    dt: float
    conductance: float
    edge_conductance: np.ndarray | None = None


def step_inputs(mesh, seed: int, edge_diffusivity: np.ndarray | None = None) -> StepInputs:
    """Inputs of one sub-step on `mesh` (a planet_game_gb300 PlanetMesh)."""
    return step_inputs_from(mesh.arrays()["center"], mesh.substep_mean_insolation(0), seed, edge_diffusivity)


def step_inputs_from(center: np.ndarray, insolation: np.ndarray, seed: int,
                     edge_diffusivity: np.ndarray | None = None) -> StepInputs:
    """The same from the cells' unit centres and the sub-step-0 mean insolation (any mesh
    builder that gives the reference's mesh gives the same inputs)."""
    rng = np.random.default_rng(seed)
    t0 = initial_temperature(center, rng)
    s = source_term(insolation, t0)
    g = None if edge_diffusivity is None else HEAT_CAPACITY * edge_diffusivity
    return StepInputs(t0, s, HEAT_CAPACITY, SUBSTEP_S, HEAT_CAPACITY * DIFFUSIVITY, g)


def perturbed_sources(source: np.ndarray, count: int, seed: int, sigma: float = 5.0) -> np.ndarray:
    """`count` right-hand sides: the source plus N(0, sigma) W/m^2 per cell."""
    rng = np.random.default_rng(seed)
    return source[None, :] + rng.normal(0.0, sigma, (count, len(source)))


def lognormal_edge_diffusivity(edges: int, seed: int, median: float = DIFFUSIVITY, sigma: float = 0.5) -> np.ndarray:
    """Per undirected edge, so the conductance is symmetric by construction."""
    rng = np.random.default_rng(seed)
    return median * np.exp(rng.normal(0.0, sigma, edges))


# ---- real spherical harmonics ------------------------------------------------------------

def _legendre(lmax: int, x: np.ndarray, s: np.ndarray):
    """Orthonormal associated Legendre functions Pbar[l][m](x) (for real Y_lm with the
    sqrt(2) cos/sin factor) and their theta derivatives, x = cos(theta), s = sin(theta) > 0."""
    n = len(x)
    P = np.zeros((lmax + 1, lmax + 1, n))
    dP = np.zeros((lmax + 1, lmax + 1, n))
    P[0, 0] = 1.0 / np.sqrt(4.0 * np.pi)
    for m in range(1, lmax + 1):
        P[m, m] = np.sqrt((2.0 * m + 1.0) / (2.0 * m)) * s * P[m - 1, m - 1]
    for m in range(0, lmax):
        P[m + 1, m] = np.sqrt(2.0 * m + 3.0) * x * P[m, m]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            a = np.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = np.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
            P[l, m] = a * (x * P[l - 1, m] - b * P[l - 2, m])
    # dP/dtheta = (l x P_lm - sqrt((2l+1)/(2l-1) (l^2 - m^2)) P_{l-1,m}) / s
    for l in range(1, lmax + 1):
        for m in range(0, l + 1):
            c = np.sqrt((2.0 * l + 1.0) / (2.0 * l - 1.0) * (l * l - m * m)) if l > m else 0.0
            prev = P[l - 1, m] if l - 1 >= m else 0.0
            dP[l, m] = (l * x * P[l, m] - c * prev) / s
    return P, dP


def real_harmonics(lmax: int, unit: np.ndarray):
    """Y[l][m + lmax] and its gradient parts at unit vectors: returns Y, dY/dtheta,
    dY/dphi / sin(theta), arrays of shape (lmax+1, 2 lmax+1, n)."""
    x = np.clip(unit[:, 2], -1.0, 1.0)
    s = np.sqrt(np.maximum(unit[:, 0] ** 2 + unit[:, 1] ** 2, 1e-300))
    phi = np.arctan2(unit[:, 1], unit[:, 0])
    P, dP = _legendre(lmax, x, s)
    n = len(x)
    Y = np.zeros((lmax + 1, 2 * lmax + 1, n))
    Yt = np.zeros_like(Y)
    Yp = np.zeros_like(Y)
    r2 = np.sqrt(2.0)
    for l in range(lmax + 1):
        Y[l, lmax] = P[l, 0]
        Yt[l, lmax] = dP[l, 0]
        for m in range(1, l + 1):
            c, sn = np.cos(m * phi), np.sin(m * phi)
            Y[l, lmax + m] = r2 * P[l, m] * c
            Y[l, lmax - m] = r2 * P[l, m] * sn
            Yt[l, lmax + m] = r2 * dP[l, m] * c
            Yt[l, lmax - m] = r2 * dP[l, m] * sn
            Yp[l, lmax + m] = -r2 * m * P[l, m] / s * sn
            Yp[l, lmax - m] = r2 * m * P[l, m] / s * c
    return Y, Yt, Yp


def harmonic_coefficients(lmax: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((lmax + 1, 2 * lmax + 1))
    for l in range(lmax + 1):
        c[l, : lmax - l] = 0.0
        c[l, lmax + l + 1:] = 0.0
    return c


@dataclass
class HarmonicField:
    value: np.ndarray           # f at cell centres
    east: np.ndarray            # analytic gradient, east component (1/m)
    north: np.ndarray           # analytic gradient, north component
    laplacian: np.ndarray       # analytic Laplacian (1/m^2)
    edge_flux: np.ndarray       # exact edge-normal flux of grad f at edge midpoints


def _gradient3(coef, lmax, unit, radius):
    Y, Yt, Yp = real_harmonics(lmax, unit)
    f = np.einsum("lm,lmn->n", coef, Y)
    ft = np.einsum("lm,lmn->n", coef, Yt)        # df/dtheta
    fp = np.einsum("lm,lmn->n", coef, Yp)        # (1/sin) df/dphi
    theta_hat_north = -1.0                        # north = -theta_hat
    east = fp / radius
    north = theta_hat_north * ft / radius
    return f, east, north, Y


def harmonic_field(mesh_arrays: dict, radius: float, lmax: int, seed: int) -> HarmonicField:
    coef = harmonic_coefficients(lmax, seed)
    center = mesh_arrays["center"]
    f, east, north, Y = _gradient3(coef, lmax, center, radius)
    ll = np.arange(lmax + 1)
    lap = np.einsum("lm,lmn->n", coef * (-(ll * (ll + 1.0)) / radius**2)[:, None], Y)
    # exact edge fluxes: endpoints CCW around the edge's first cell
    first = mesh_arrays["edge_first"]
    off = mesh_arrays["edge_offset"].astype(np.int64)
    cnt = mesh_arrays["edge_count"].astype(np.int64)
    ncells = len(off)
    rows = np.repeat(np.arange(ncells), cnt)
    local = np.arange(len(rows)) - off[rows]
    nxt = off[rows] + (local + 1) % cnt[rows]
    owner = first[mesh_arrays["edge"]] == rows
    e_of = mesh_arrays["edge"][owner]
    c1 = mesh_arrays["corner"][owner]
    c2 = mesh_arrays["corner"][nxt[owner]]
    corners = mesh_arrays["corner_unit"]
    p1, p2 = corners[c1], corners[c2]
    normal = np.cross(p1, p2)
    normal /= np.linalg.norm(normal, axis=1)[:, None]
    flip = np.einsum("ij,ij->i", normal, center[first[e_of]]) > 0.0
    normal[flip] *= -1.0
    mid = p1 + p2
    mid /= np.linalg.norm(mid, axis=1)[:, None]
    _, e_m, n_m, _ = _gradient3(coef, lmax, mid, radius)
    # local basis at the midpoints: east = (-y, x, 0)/h, north = up x east
    h = np.sqrt(mid[:, 0] ** 2 + mid[:, 1] ** 2)
    east_hat = np.stack([-mid[:, 1] / h, mid[:, 0] / h, np.zeros(len(mid))], axis=1)
    north_hat = np.cross(mid, east_hat)
    grad3 = e_m[:, None] * east_hat + n_m[:, None] * north_hat
    flux = np.empty(len(first))
    flux[e_of] = np.einsum("ij,ij->i", grad3, normal)
    return HarmonicField(f, east, north, lap, flux)


# ---- column radiation inputs ------------------------------------------------------------------

R_DRY = 287.04
EPSILON = R_DRY / 461.5


def saturation_vapour_pressure(t: np.ndarray) -> np.ndarray:
    """Bolton (1980) over water at and above 0 C, Murphy-Koop (2005) over ice below it,
    scaled to meet at 0 C (the reference's saturation.cpp)."""
    t = np.asarray(t, dtype=np.float64)

    def mk(x):
        return np.exp(9.550426 - 5723.265 / x + 3.53068 * np.log(x) - 0.00728332 * x)

    water = 611.2 * np.exp(17.67 * (t - 273.15) / (t - 29.65))
    ice = 611.2 / mk(273.15) * mk(t)
    return np.where(t >= 273.15, water, ice)


def saturation_specific_humidity(t: np.ndarray, p: np.ndarray) -> np.ndarray:
    e = saturation_vapour_pressure(t)
    den = p - (1.0 - EPSILON) * e
    return np.where(den > EPSILON * e, EPSILON * e / np.where(den > 0, den, 1.0), 1.0)


@dataclass
class ColumnInputs:
    temperature: np.ndarray     # [layers, cells]
    humidity: np.ndarray
    cloud_water: np.ndarray
    surface_temperature: np.ndarray
    surface_pressure: np.ndarray
    cloud_fraction: np.ndarray


def column_profiles(surface_temperature: np.ndarray, layers: int, seed: int, lapse_K_m: float = 6.5e-3,
                    surface_pressure_Pa: float = 1.0e5, relative_humidity: float = 0.8) -> ColumnInputs:
    rng = np.random.default_rng(seed)
    n = len(surface_temperature)
    sigma = 1.0 - (np.arange(layers) + 0.5) / layers
    p = sigma[:, None] * surface_pressure_Pa * np.ones((1, n))
    # constant lapse rate: T = Ts (p/ps)^(R_d Gamma / g), i.e. Ts - Gamma z with z hypsometric
    temp = surface_temperature[None, :] * sigma[:, None] ** (R_DRY * lapse_K_m / EARTH_GRAVITY)
    q = relative_humidity * saturation_specific_humidity(temp, p)
    f = rng.random((layers, n))
    mass = surface_pressure_Pa / (EARTH_GRAVITY * layers)
    ql = f * EARTH_COLUMN["in_cloud_water_path_kg_m2"] / mass
    return ColumnInputs(temp, q, ql, surface_temperature.copy(), np.full(n, surface_pressure_Pa), f)


def column_constant_vector(c: dict = EARTH_COLUMN) -> np.ndarray:
    keys = ("dry_optical_depth", "vapour_absorption_m2_kg", "in_cloud_water_path_kg_m2", "effective_radius_m",
            "cloud_asymmetry", "cloud_longwave_absorption_m2_kg", "reference_pressure_Pa", "gravity_m_s2",
            "stefan_boltzmann")
    return np.array([c[k] for k in keys])


# ---- batched and served workloads ----------------------------------------------------------------

PLANET_MIX = ((4, 16), (5, 24), (6, 16), (7, 8))   # 64 planets, 2,252,928 cells


@dataclass
class PlanetSpec:
    level: int
    radius: float
    seed: int


def planet_mix(seed: int, mix=PLANET_MIX) -> list[PlanetSpec]:
    rng = np.random.default_rng(seed)
    specs = []
    for level, count in mix:
        for _ in range(count):
            specs.append(PlanetSpec(level, float(rng.uniform(3e6, 9e6)), int(rng.integers(0, 2**31))))
    return specs


@dataclass
class Request:
    arrival_s: float
    level: int
    planet: int


def poisson_trace(count: int, rate_per_s: float, seed: int, weights=((4, .30), (5, .30), (6, .20), (7, .15), (8, .05)),
                  planets_per_level: int = 4) -> list[Request]:
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, count)
    levels = np.array([w[0] for w in weights])
    p = np.array([w[1] for w in weights])
    lv = rng.choice(levels, size=count, p=p / p.sum())
    pl = rng.integers(0, planets_per_level, count)
    t = np.cumsum(gaps)
    return [Request(float(t[i]), int(lv[i]), int(pl[i])) for i in range(count)]


# ---- non-symmetric transport cases (tracer, coupled advection-diffusion) -----------------

def reverse_entries(offset: np.ndarray, neighbour: np.ndarray) -> np.ndarray:
    """For every CSR entry a -> b, the entry b -> a."""
    offset = offset.astype(np.int64)
    neighbour = neighbour.astype(np.int64)
    rows = np.repeat(np.arange(len(offset) - 1), np.diff(offset))
    # entries sorted by (row, neighbour) and by (neighbour, row) pair up one to one
    forward = np.lexsort((neighbour, rows))
    backward = np.lexsort((rows, neighbour))
    rev = np.empty(len(neighbour), dtype=np.int64)
    rev[forward] = backward
    return rev


def antisymmetric_layer_fluxes(offset, neighbour, layers: int, scale: float, seed: int,
                               column_balanced: bool = True) -> np.ndarray:
    """Layer mass fluxes per CSR entry (kg/s, layer-major) of about `scale`, antisymmetric
    per face; with `column_balanced` each face's column sums to zero (the shape of the
    reference's transport tests, test_tracer_transport.cpp:33-60)."""
    offset = offset.astype(np.int64)
    neighbour = neighbour.astype(np.int64)
    rows = np.repeat(np.arange(len(offset) - 1), np.diff(offset))
    upper = np.nonzero(rows < neighbour)[0]
    rev = reverse_entries(offset, neighbour)
    rng = np.random.default_rng(seed)
    flow = scale * (2.0 * rng.random((layers, len(upper))) - 1.0)
    if column_balanced:
        flow -= flow.mean(axis=0, keepdims=True)
    out = np.zeros((layers, len(neighbour)))
    out[:, upper] = flow
    out[:, rev[upper]] = -flow
    return out.ravel()


def agglomerated_step_inputs(nodes: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """T0 = 288 + N(0, 0.5) K and S = N(0, 50) W/m^2 per node: the transport step on an
    agglomerated graph (nodes of the coarser mesh)."""
    rng = np.random.default_rng(seed)
    return 288.0 + rng.normal(0.0, 0.5, nodes), rng.normal(0.0, 50.0, nodes)


def tracer_field(count: int, seed: int) -> np.ndarray:
    """Positive mixing ratios around 0.01 (layer-major)."""
    return 0.01 * (1.0 + 0.5 * np.random.default_rng(seed).standard_normal(count) ** 2)


def quartic_column(a: float, radiative: float, nodes: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """The reference test's quartic column (test_heat_transport.cpp:58-76): forcings b
    putting each column's equilibrium between 200 and 320 K, and the floor of sources
    that keeps every column at or above 100 K."""
    target = 200.0 + 120.0 * np.random.default_rng(seed).random(nodes)
    b = a * target + radiative * target ** 4
    return b, a * 100.0 + radiative * 100.0 ** 4 - b
