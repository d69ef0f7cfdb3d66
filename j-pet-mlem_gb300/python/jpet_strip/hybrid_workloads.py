"""Synthetic inputs of the 3D hybrid reconstruction: a one-ring barrel's LOR
geometry (the arrays of PET2D::Barrel::GeometrySOA, src/2d/barrel/geometry_soa.h:
268-283) and list-mode responses of a 3D ellipsoid phantom in the hybrid
scanner's Response layout (src/3d/hybrid/scanner.h:71-87).

The reference reads its geometry from a barrel geometry or system-matrix file
made by its Monte Carlo matrix tools; neither tool is part of this path, so a
deterministic construction stands in: detectors evenly on a circle, each LOR the
segment between two detector centres (LineSegment(c[second], c[first]) as the
geometry constructor builds it, geometry_soa.h:120-124), its pixel infos the grid
pixels whose centres lie within the LOR width of the line and between the two
detectors, ordered by their scaled projection along the LOR (:126-137).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

f32 = np.float32

SEGMENT_DTYPE = np.dtype([(n, "<f4") for n in (
    "start_x", "start_y", "end_x", "end_y", "mid_x", "mid_y", "dir_x", "dir_y", "normal_x",
    "normal_y", "length", "distance_from_origin")])
PIXEL_DTYPE = np.dtype([("x", "<i2"), ("y", "<i2")])
RESPONSE_DTYPE = np.dtype([("first", "<i2"), ("second", "<i2"), ("z_up", "<f4"),
                           ("z_dn", "<f4"), ("dl", "<f4")])
FRAME_EVENT_DTYPE = np.dtype({
    "names": ["first", "second", "up", "right", "tan", "sec", "info_begin", "info_end",
              "plane_begin", "plane_end"],
    "formats": ["<i2", "<i2", "<f4", "<f4", "<f4", "<f4", "<u8", "<u8", "<i2", "<i2"],
    "offsets": [0, 2, 4, 8, 12, 16, 24, 32, 40, 42],
    "itemsize": 48})


@dataclass
class HybridGeometry:
    n_detectors: int
    segments: np.ndarray       # SEGMENT_DTYPE[n_lors]
    widths: np.ndarray         # float32[n_lors]
    pixels: np.ndarray         # PIXEL_DTYPE[n_infos]
    positions: np.ndarray      # float32[n_infos]
    weights: np.ndarray        # float32[n_planes_half * n_infos] (system-matrix weights,
                               # plane-major; zeros = computed)
    info_begin: np.ndarray     # uint64[n_lors]
    info_end: np.ndarray       # uint64[n_lors]
    n_columns: int
    n_rows: int
    n_planes: int
    pixel_size: float
    lower_left_x: float
    lower_left_y: float
    z_left: float
    sigma_z: float
    sigma_dl: float
    length: float
    radius: float
    n_planes_half: int = 1     # planes of weights (> 1: one system matrix per plane half)

    @property
    def n_lors(self) -> int:
        return (self.n_detectors + 1) * self.n_detectors // 2

    @property
    def n_pixel_infos(self) -> int:
        return int(self.pixels.shape[0])

    @property
    def n_voxels(self) -> int:
        return self.n_columns * self.n_rows * self.n_planes


def _segment(sx, sy, ex, ey):
    """LineSegment(start, end) fields in float32 as its constructor computes
    them (src/2d/geometry/line_segment.h:27-34, vector.h:56-72,96,127)."""
    sx, sy, ex, ey = (np.asarray(v, f32) for v in (sx, sy, ex, ey))
    mx = (sx + ex) / f32(2)
    my = (sy + ey) / f32(2)
    dx = ex - sx
    dy = ey - sy
    ln = np.sqrt(dx * dx + dy * dy)
    with np.errstate(invalid="ignore", divide="ignore"):
        ux = np.where(ln > 0, dx / ln, f32(0)).astype(f32)
        uy = np.where(ln > 0, dy / ln, f32(0)).astype(f32)
    nx, ny = -uy, ux
    dfo = sx * nx + sy * ny
    return mx, my, ux, uy, nx, ny, ln, dfo


def ring_geometry(n_detectors: int, radius: float, width: float, n_pixels: int,
                  pixel_size: float, n_planes: int, sigma_z: float, sigma_dl: float,
                  length: float, band: float | None = None, weights: str = "computed",
                  seed: int = 0) -> HybridGeometry:
    """One ring of n_detectors on a circle of the given radius; LOR width
    `width`; pixel infos within `band` (default: the width) of each LOR line.
    weights: "computed" (zeros; the reconstruction computes them from the
    widths) or "given" (seeded positive system-matrix-like weights)."""
    band = width if band is None else band
    ang = 2 * np.pi * np.arange(n_detectors) / n_detectors
    cx = (radius * np.cos(ang)).astype(f32)
    cy = (radius * np.sin(ang)).astype(f32)
    first = np.concatenate([np.full(i + 1, i) for i in range(n_detectors)])
    second = np.concatenate([np.arange(i + 1) for i in range(n_detectors)])
    n_lors = first.shape[0]
    seg = np.zeros(n_lors, SEGMENT_DTYPE)
    seg["start_x"], seg["start_y"] = cx[second], cy[second]
    seg["end_x"], seg["end_y"] = cx[first], cy[first]
    (seg["mid_x"], seg["mid_y"], seg["dir_x"], seg["dir_y"], seg["normal_x"], seg["normal_y"],
     seg["length"], seg["distance_from_origin"]) = _segment(cx[second], cy[second], cx[first],
                                                           cy[first])
    ps = f32(pixel_size)
    llx = f32(f32(-ps * f32(n_pixels)) / f32(2))
    lly = llx
    llcx = f32(llx + ps / f32(2))
    # candidate pixels per LOR: all pixels of the LOR's bounding box widened by the band
    pixels, positions, begin, end = [], [], np.zeros(n_lors, np.uint64), np.zeros(n_lors, np.uint64)
    idx = np.arange(n_pixels)
    centers = (llcx + idx.astype(f32) * ps).astype(np.float64)
    total = 0
    for l in range(n_lors):
        begin[l] = total
        if first[l] == second[l]:
            end[l] = total
            continue
        s = seg[l]
        x0, x1 = sorted((float(s["start_x"]), float(s["end_x"])))
        y0, y1 = sorted((float(s["start_y"]), float(s["end_y"])))
        ix = idx[(centers >= x0 - band) & (centers <= x1 + band)]
        iy = idx[(centers >= y0 - band) & (centers <= y1 + band)]
        if ix.size == 0 or iy.size == 0:
            end[l] = total
            continue
        # the line's distance is linear in x and y: keep a thin stripe only
        px = centers[ix][:, None]
        py = centers[iy][None, :]
        dist = px * float(s["normal_x"]) + py * float(s["normal_y"]) - float(
            s["distance_from_origin"])
        t = ((px - float(s["start_x"])) * float(s["dir_x"]) +
             (py - float(s["start_y"])) * float(s["dir_y"])) / float(s["length"])
        keep = (np.abs(dist) <= band) & (t >= 0) & (t <= 1)
        kx, ky = np.nonzero(keep)
        if kx.size == 0:
            end[l] = total
            continue
        gx, gy = ix[kx], iy[ky]
        # scaled projection in float32 as projection_scaled computes it (line_segment.h:72-77)
        cxf = (llcx + gx.astype(f32) * ps).astype(f32)
        cyf = (llcx + gy.astype(f32) * ps).astype(f32)
        proj = ((cxf - s["start_x"]) * s["dir_x"] + (cyf - s["start_y"]) * s["dir_y"]).astype(f32)
        pos = (proj / s["length"]).astype(f32)
        order = np.argsort(pos, kind="stable")
        p = np.empty(order.size, PIXEL_DTYPE)
        p["x"], p["y"] = gx[order], gy[order]
        pixels.append(p)
        positions.append(pos[order])
        total += order.size
        end[l] = total
    pixels = np.concatenate(pixels) if pixels else np.zeros(0, PIXEL_DTYPE)
    positions = np.concatenate(positions).astype(f32) if positions else np.zeros(0, f32)
    if weights == "given":
        w = np.random.default_rng(seed).uniform(0.05, 1.0, pixels.shape[0]).astype(f32)
    else:
        w = np.zeros(pixels.shape[0], f32)
    z_left = f32(-n_planes * pixel_size / 2)
    return HybridGeometry(n_detectors, seg, np.full(n_lors, width, f32), pixels, positions, w,
                          begin, end, n_pixels, n_pixels, n_planes, float(ps), float(llx),
                          float(lly), float(z_left), float(f32(sigma_z)), float(f32(sigma_dl)),
                          float(f32(length)), radius)


def ellipsoid_phantom(radius: float, length: float, seed: int = 1, n: int = 6):
    """Seeded ellipsoids (centre, semi-axes, intensity) inside the field of view."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        r = rng.uniform(0, 0.5 * radius)
        a = rng.uniform(0, 2 * np.pi)
        c = (r * np.cos(a), r * np.sin(a), rng.uniform(-0.3, 0.3) * length)
        ax = (rng.uniform(0.05, 0.2) * radius, rng.uniform(0.05, 0.2) * radius,
              rng.uniform(0.05, 0.15) * length)
        out.append((c, ax, rng.uniform(0.5, 2.0)))
    return out


def responses(geom: HybridGeometry, n: int, seed: int = 2, phantom=None,
              max_tan: float = 1.0) -> np.ndarray:
    """n detected responses (RESPONSE_DTYPE) of emissions in the phantom: an
    emission point, an in-plane direction and an axial slope; the LOR is the
    pair of detectors nearest to where the line meets the ring; z_up, z_dn and
    dl are the exact values along that LOR plus Gaussian noise of sigma_z,
    sigma_z and sigma_dl.  Emissions whose line leaves the scanner length are
    not detected."""
    rng = np.random.default_rng(seed)
    phantom = phantom or ellipsoid_phantom(geom.radius, geom.length, seed + 1)
    weights = np.array([p[2] * np.prod(p[1]) for p in phantom])
    weights /= weights.sum()
    out = np.zeros(0, RESPONSE_DTYPE)
    N, R0, half = geom.n_detectors, geom.radius, geom.length / 2
    while out.shape[0] < n:
        m = int((n - out.shape[0]) * 1.5) + 1024
        k = rng.choice(len(phantom), m, p=weights)
        u = rng.normal(size=(m, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        rad = rng.uniform(0, 1, m) ** (1 / 3)
        c = np.array([phantom[i][0] for i in k])
        ax = np.array([phantom[i][1] for i in k])
        p = c + u * rad[:, None] * ax
        phi = rng.uniform(0, np.pi, m)
        tn = rng.uniform(-max_tan, max_tan, m)
        d = np.stack([np.cos(phi), np.sin(phi)], 1)
        pd = np.sum(p[:, :2] * d, 1)
        disc = pd * pd - np.sum(p[:, :2] ** 2, 1) + R0 * R0
        ok = disc > 0
        sq = np.sqrt(np.where(ok, disc, 0))
        q1 = p[:, :2] + d * (-pd + sq)[:, None]
        q2 = p[:, :2] + d * (-pd - sq)[:, None]
        i1 = np.mod(np.rint(np.arctan2(q1[:, 1], q1[:, 0]) / (2 * np.pi / N)), N).astype(np.int64)
        i2 = np.mod(np.rint(np.arctan2(q2[:, 1], q2[:, 0]) / (2 * np.pi / N)), N).astype(np.int64)
        ok &= i1 != i2
        f = np.maximum(i1, i2)
        s = np.minimum(i1, i2)
        lor = f * (f + 1) // 2 + s
        sg = geom.segments[lor]
        upv = (p[:, 0] - sg["mid_x"]) * sg["dir_x"] + (p[:, 1] - sg["mid_y"]) * sg["dir_y"]
        Rl = sg["length"].astype(np.float64) / 2
        z0 = p[:, 2]
        z_up = z0 + (Rl - upv) * tn
        z_dn = z0 - (Rl + upv) * tn
        ok &= (np.abs(z_up) <= half) & (np.abs(z_dn) <= half) & (np.abs(upv) < Rl)
        dl = -2 * upv * np.sqrt(1 + tn * tn)
        r = np.zeros(m, RESPONSE_DTYPE)
        r["first"], r["second"] = f, s
        r["z_up"] = z_up + rng.normal(0, geom.sigma_z, m)
        r["z_dn"] = z_dn + rng.normal(0, geom.sigma_z, m)
        r["dl"] = dl + rng.normal(0, geom.sigma_dl, m)
        out = np.concatenate([out, r[ok]])
    return out[:n].copy()


# Named configurations (lengths in metres as the reference's hybrid tools use
# them; sigma_z / sigma_dl are 3d_hybrid_reconstruction's defaults, 0.015 / 0.060).
HYBRID_WORKLOADS = {
    # golden-vector case: small enough for the reference harness in seconds
    "hybrid-tiny": dict(n_detectors=24, radius=0.25, width=0.02, n_pixels=24,
                        pixel_size=0.02, n_planes=12, sigma_z=0.015, sigma_dl=0.060,
                        length=0.24, n_events=400, iterations=3),
    # parity case for the GPU tests
    "hybrid-96": dict(n_detectors=96, radius=0.43, width=0.012, n_pixels=100,
                      pixel_size=0.008, n_planes=60, sigma_z=0.015, sigma_dl=0.060,
                      length=0.48, n_events=200_000, iterations=5),
    # benchmark case: 384-detector ring, 4 mm voxels over 0.8 x 0.8 x 0.5 m
    "hybrid-384": dict(n_detectors=384, radius=0.43, width=0.007, n_pixels=200,
                       pixel_size=0.004, n_planes=125, sigma_z=0.015, sigma_dl=0.060,
                       length=0.5, n_events=10_000_000, iterations=10),
}


def workload(name: str, weights: str = "computed"):
    """(geometry, n_events, iterations) of a named configuration."""
    w = dict(HYBRID_WORKLOADS[name])
    n, it = w.pop("n_events"), w.pop("iterations")
    return ring_geometry(weights=weights, **w), n, it


def from_arrays(d, prefix: str = "") -> HybridGeometry:
    """HybridGeometry from a mapping of arrays as tests/golden/hybrid_ref.npz
    stores them (keys <prefix>segments, ..., <prefix>grid, <prefix>params)."""
    gi = d[prefix + "grid"]
    pa = d[prefix + "params"]
    h = int(gi[7]) if gi.shape[0] > 7 else 1
    return HybridGeometry(int(gi[0]), d[prefix + "segments"], d[prefix + "widths"],
                          d[prefix + "pixels"], d[prefix + "positions"],
                          d[prefix + "weights_in"], d[prefix + "info_begin"],
                          d[prefix + "info_end"], int(gi[1]), int(gi[2]), int(gi[3]),
                          *[float(v) for v in pa], n_planes_half=h)


def multiplane_weights(g: HybridGeometry, n_planes_half: int, seed: int = 0) -> HybridGeometry:
    """The geometry with n_planes_half planes of seeded system-matrix weights
    (what 3d_hybrid_reconstruction loads from one --system matrix per plane
    half, reconstruction_cmd.cpp:340-358): plane 0 the given weights, plane k
    those weights times a seeded factor in [0.5, 1.5) per info."""
    import dataclasses

    rng = np.random.default_rng(seed)
    w0 = np.asarray(g.weights, f32)[:g.n_pixel_infos]
    planes = [w0] + [(w0 * rng.uniform(0.5, 1.5, w0.shape[0])).astype(f32)
                     for _ in range(1, n_planes_half)]
    return dataclasses.replace(g, weights=np.concatenate(planes).astype(f32),
                               n_planes_half=n_planes_half)
