"""Seeded synthetic list-mode event generator for the 2D strip scanner.

Follows the reference phantom tool's generator semantics
(``src/2d/strip/phantom_cmd.cpp:136-444``, ``src/common/phantom_monte_carlo.h:33-109``):

1. a region is chosen with probability intensity x area
   (``src/2d/geometry/phantom.h:57,120-133,183-191``);
2. a uniform point is drawn in the ellipse with ``r = sqrt(U)``, ``theta = 2 pi U``
   (``src/2d/geometry/ellipse.h:83-91``); regions are disjunctive: a point that
   lies in an earlier-listed region is redrawn (``phantom.h:193-204``), unless
   ``additive`` is set;
3. the emission angle is uniform; the reference draws it in (-pi/2, pi/2)
   (``phantom.h:213``) and keeps only detected events.  Every detected event has
   ``|tan| < L / 2R`` because ``|z_u - z_d| = 2R |tan| < L``, so drawing the angle
   uniformly in ``+-atan(L / 2R)`` gives the same distribution of accepted events
   with fewer rejections;
4. the line is intersected with both strips (``src/2d/strip/scanner.h:107-113``),
   direction ``(sin phi, cos phi)`` so ``tan = tan(phi)`` (``src/2d/geometry/event.h:39-40``);
5. the event is accepted iff ``|z_u|, |z_d| < L/2`` on the exact values
   (``scanner.h:208-213``);
6. ``z_u``, ``z_d`` are smeared by N(0, sigma_z) and ``dl`` by N(0, sigma_dl)
   with no re-rejection (``scanner.h:257-267``).

Random numbers come from numpy's counter-based Philox generator, seeded per
workload, so a given (phantom, scanner, n, seed) always yields the same events.
Output is float32 AoS triples ``(z_u, z_d, dl)``, the reference binary response
format (``src/2d/strip/reconstruction.h:156-167``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Ellipse:
    """Phantom ellipse: centre (z, y), semi-axes a (along z) and b, rotation in
    degrees, intensity -- the ``ellipse x y a b angle intensity`` line of the
    reference phantom format (``src/2d/geometry/phantom.h:137-181``)."""

    z: float
    y: float
    a: float
    b: float
    angle_deg: float
    intensity: float

    @property
    def area(self) -> float:
        return math.pi * self.a * self.b

    def contains(self, z: np.ndarray, y: np.ndarray) -> np.ndarray:
        # Ellipse::contains (src/2d/geometry/ellipse.h:32-35)
        ang = math.radians(self.angle_deg)
        s, c = math.sin(ang), math.cos(ang)
        A = c * c / (self.a * self.a) + s * s / (self.b * self.b)
        B = s * s / (self.a * self.a) + c * c / (self.b * self.b)
        C = s * c * (1 / (self.a * self.a) - 1 / (self.b * self.b))
        rz, ry = z - self.z, y - self.y
        return A * rz * rz + 2 * C * rz * ry + B * ry * ry <= 1


def parse_phantom(text: str, scale: float = 1.0) -> list[Ellipse]:
    """Parses ``ellipse x y a b angle intensity`` lines (phantom.h:137-181)."""
    out = []
    for line in text.splitlines():
        parts = line.split()
        if not parts or parts[0].startswith("#"):
            continue
        if parts[0] != "ellipse":
            raise ValueError(f"unsupported phantom region: {parts[0]}")
        x, y, a, b, ang, inten = (float(v) for v in parts[1:7])
        out.append(Ellipse(x * scale, y * scale, a * scale, b * scale, ang, inten))
    return out


def generate_events(
    ellipses: list[Ellipse],
    n_events: int,
    radius: float,
    length: float,
    sigma_z: float,
    sigma_dl: float,
    seed: int,
    additive: bool = False,
    batch: int = 1 << 21,
) -> np.ndarray:
    """Returns float32[n_events, 3] detected and smeared responses (z_u, z_d, dl)."""
    rng = np.random.Generator(np.random.Philox(seed))
    weights = np.array([e.intensity * e.area for e in ellipses], dtype=np.float64)
    cdf = np.cumsum(weights) / weights.sum()
    tan_max = length / (2.0 * radius)
    phi_max = math.atan(tan_max)
    out = np.empty((n_events, 3), dtype=np.float32)
    filled = 0
    while filled < n_events:
        m = batch
        region = np.searchsorted(cdf, rng.random(m), side="left")
        region = np.minimum(region, len(ellipses) - 1)
        u_ang = rng.random(m)
        u_r = rng.random(m)
        theta = 2.0 * math.pi * u_ang
        r = np.sqrt(u_r)
        za = np.empty(m)
        ya = np.empty(m)
        keep = np.ones(m, dtype=bool)
        for i, e in enumerate(ellipses):
            sel = region == i
            if not sel.any():
                continue
            ang = math.radians(e.angle_deg)
            s, c = math.sin(ang), math.cos(ang)
            x = e.a * r[sel] * np.cos(theta[sel])
            yy = e.b * r[sel] * np.sin(theta[sel])
            za[sel] = c * x - s * yy + e.z
            ya[sel] = s * x + c * yy + e.y
        if not additive:
            for i, e in enumerate(ellipses):
                sel = region > i
                if sel.any():
                    inside = np.zeros(m, dtype=bool)
                    inside[sel] = e.contains(za[sel], ya[sel])
                    keep &= ~inside
        phi = phi_max * (2.0 * rng.random(m) - 1.0)
        t = np.tan(phi)
        z_u = za + (radius - ya) * t
        z_d = za - (radius + ya) * t
        dl = -2.0 * ya * np.sqrt(t * t + 1.0)
        half = length / 2.0
        keep &= (np.abs(z_u) < half) & (np.abs(z_d) < half)
        noise = rng.standard_normal((m, 3))
        idx = np.nonzero(keep)[0]
        take = min(len(idx), n_events - filled)
        idx = idx[:take]
        out[filled : filled + take, 0] = z_u[idx] + sigma_z * noise[idx, 0]
        out[filled : filled + take, 1] = z_d[idx] + sigma_z * noise[idx, 1]
        out[filled : filled + take, 2] = dl[idx] + sigma_dl * noise[idx, 2]
        filled += take
    return out


# --- workload phantoms -------------------------------------------------------------

def three_ellipse_phantom() -> list[Ellipse]:
    """Three-ellipse phantom of the 5 mm plain workload (hot region listed first)."""
    return [
        Ellipse(120.0, -40.0, 150.0, 150.0, 0.0, 2.0),
        Ellipse(-100.0, 50.0, 180.0, 150.0, 30.0, 0.5),
        Ellipse(0.0, 0.0, 300.0, 250.0, 0.0, 1.0),
    ]


def _fit_ellipse(z, y, a, b, ang_deg, half_z, half_y):
    ang = math.radians(ang_deg)
    ez = math.sqrt((a * math.cos(ang)) ** 2 + (b * math.sin(ang)) ** 2)
    ey = math.sqrt((a * math.sin(ang)) ** 2 + (b * math.cos(ang)) ** 2)
    room_z = half_z - abs(z)
    room_y = half_y - abs(y)
    f = min(1.0, room_z / ez, room_y / ey)
    return a * f, b * f


def random_ellipse_phantom(
    seed: int,
    n: int = 10,
    half_z: float = 500.0,
    half_y: float = 450.0,
    centre_z: float = 300.0,
    centre_y: float = 250.0,
    axes: tuple[float, float] = (20.0, 350.0),
    intensity: tuple[float, float] = (0.1, 2.0),
) -> list[Ellipse]:
    """Seeded Shepp-Logan-like phantom: centres uniform in |z|<=centre_z,
    |y|<=centre_y, semi-axes U[axes] shrunk to fit the field of view, rotation
    U[0, 180) degrees, intensity U[intensity].  Listed smallest first, so nested
    small structures take precedence under the disjunctive rule."""
    rng = np.random.Generator(np.random.Philox(seed))
    out = []
    for _ in range(n):
        z = rng.uniform(-centre_z, centre_z)
        y = rng.uniform(-centre_y, centre_y)
        a = rng.uniform(*axes)
        b = rng.uniform(*axes)
        ang = rng.uniform(0.0, 180.0)
        inten = rng.uniform(*intensity)
        a, b = _fit_ellipse(z, y, a, b, ang, half_z, half_y)
        out.append(Ellipse(z, y, a, b, ang, inten))
    out.sort(key=lambda e: e.area)
    return out


def lesion_phantom(seed: int, n_background: int = 10, n_lesions: int = 6,
                   lesion_radius: float = 5.0, contrast: float = 8.0) -> list[Ellipse]:
    """Background of random ellipses plus hot circular lesions of the given radius
    at ``contrast`` times the intensity of the region they sit in."""
    bg = random_ellipse_phantom(seed, n_background)
    rng = np.random.Generator(np.random.Philox(seed + 1000))
    lesions = []
    big = max(bg, key=lambda e: e.area)
    for _ in range(n_lesions):
        for _try in range(100):
            z = rng.uniform(-250.0, 250.0)
            y = rng.uniform(-200.0, 200.0)
            if big.contains(np.array([z]), np.array([y]))[0]:
                break
        host = [e for e in bg if e.contains(np.array([z]), np.array([y]))[0]]
        base = host[0].intensity if host else big.intensity
        lesions.append(Ellipse(z, y, lesion_radius, lesion_radius, 0.0, contrast * base))
    return lesions + bg


def point_source(z: float = -1.0, y: float = -1.0, radius: float = 0.3) -> list[Ellipse]:
    """Calibration source: one disc of the given radius (mm) at (z, y); the
    default sits on the centre of the 2 mm pixel next to the middle of the
    500 x 450 field of view."""
    return [Ellipse(z, y, radius, radius, 0.0, 1.0)]


def point_image(n_y: int, n_z: int, pixel: float, points) -> np.ndarray:
    """float32[n_y, n_z] image with unit mass in the pixel holding each (z, y);
    pixel (iy, iz) has its centre at z = (iz + 0.5) p - n_z p / 2,
    y = n_y p / 2 - (iy + 0.5) p (``src/2d/strip/scanner.h:59-66,136-139``)."""
    img = np.zeros((n_y, n_z), np.float32)
    for z, y in points:
        iz = int(math.floor((z + n_z * pixel / 2) / pixel))
        iy = int(math.floor((n_y * pixel / 2 - y) / pixel))
        img[iy, iz] += 1.0
    return img
