"""Named synthetic workloads of the strip MLEM path (shapes, sizes and value
distributions of the benchmark configurations; the reference publishes no
dataset, so seeded synthetic events stand in)."""
from __future__ import annotations

from dataclasses import dataclass, field

from . import phantom


@dataclass(frozen=True)
class Workload:
    name: str
    radius: float
    length: float
    n_y: int
    n_z: int
    pixel: float
    sigma_z: float
    sigma_dl: float
    n_events: int
    iterations: int
    seed: int
    phantom: str = "random10"
    extra: dict = field(default_factory=dict)

    def ellipses(self):
        if self.phantom == "three":
            return phantom.three_ellipse_phantom()
        if self.phantom == "lesions":
            return phantom.lesion_phantom(self.seed)
        return phantom.random_ellipse_phantom(self.seed)

    def events(self, n: int | None = None, device: int | None = 0):
        """Detected responses float32[n, 3].  With a CUDA device the GPU generator
        (capi.generate) draws them; without one, the seeded CPU generator (the
        same distribution, another random stream)."""
        n = n or self.n_events
        if device is not None:
            try:
                import torch

                if torch.cuda.is_available():
                    from . import capi

                    return capi.generate(self.ellipses(), n, self.radius, self.length,
                                         self.sigma_z, self.sigma_dl, seed=self.seed,
                                         device=device)
            except ImportError:
                pass
        return phantom.generate_events(self.ellipses(), n, self.radius, self.length,
                                       self.sigma_z, self.sigma_dl, seed=self.seed)

    def geometry_args(self):
        return (self.radius, self.length, self.n_y, self.n_z, self.pixel, self.sigma_z,
                self.sigma_dl)


def batch_instances(k: int = 64, seed0: int = 100, max_events: int = 5_000_000,
                    min_events: int = 10_000):
    """The batched workload: k independent reconstructions with seeds seed0..,
    event counts log-uniform in [min_events, max_events], grids of n_z in
    100..500 by n_y in 100..450 pixels at 2..5 mm, sigma_z in [6, 14] mm,
    sigma_dl in [30, 60] mm and 1..10 random ellipses inside the part of the
    grid the scanner sees.  Returns [(Workload, ellipses)]."""
    import numpy as np

    out = []
    for i in range(k):
        rng = np.random.default_rng(seed0 + i)
        p = float(rng.integers(2, 6))
        n_z = int(rng.integers(100, 501))
        n_y = int(rng.integers(100, 451))
        sz = float(rng.uniform(6.0, 14.0))
        sdl = float(rng.uniform(30.0, 60.0))
        n = int(np.exp(rng.uniform(np.log(min_events), np.log(max_events))))
        hz, hy = min(n_z * p / 2, 500.0), min(n_y * p / 2, 450.0)
        ell = phantom.random_ellipse_phantom(seed0 + i, n=int(rng.integers(1, 11)), half_z=hz,
                                             half_y=hy, centre_z=0.6 * hz, centre_y=0.6 * hy,
                                             axes=(10.0, 0.8 * min(hz, hy)))
        wl = Workload(f"batch-{i}", 450.0, 1000.0, n_y, n_z, p, sz, sdl, n, 10, seed0 + i,
                      "custom")
        out.append((wl, ell))
    return out


WORKLOADS = {
    # 5 mm plain CPU-runnable case: 200 x 180, 1e6 events, 3-ellipse phantom, 10 iterations
    "plain-5mm-1M": Workload("plain-5mm-1M", 450.0, 1000.0, 180, 200, 5.0, 10.0, 42.0,
                             1_000_000, 10, 1, "three"),
    # full-size plain GPU case: 500 x 450 at 2 mm, 2e7 events, 10 ellipses, 20 iterations
    "plain-2mm-20M": Workload("plain-2mm-20M", 450.0, 1000.0, 450, 500, 2.0, 10.0, 42.0,
                              20_000_000, 20, 2, "random10"),
    # the full-size case cropped to a quarter of its area with a quarter of its
    # events (the same event density per pixel, which sets how alike
    # neighbouring events are): a small case for profiles
    "plain-2mm-5M-crop": Workload("plain-2mm-5M-crop", 450.0, 1000.0, 225, 250, 2.0, 10.0,
                                  42.0, 5_000_000, 20, 2, "random10"),
    # precision stress: 1000 x 900 at 1 mm, sigma 5 / 20, lesions at 8x, 1e8 events
    "stress-1mm-100M": Workload("stress-1mm-100M", 450.0, 1000.0, 900, 1000, 1.0, 5.0, 20.0,
                                100_000_000, 30, 5, "lesions"),
}
