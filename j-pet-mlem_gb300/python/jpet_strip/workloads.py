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

    def events(self, n: int | None = None):
        return phantom.generate_events(self.ellipses(), n or self.n_events, self.radius,
                                       self.length, self.sigma_z, self.sigma_dl, seed=self.seed)

    def geometry_args(self):
        return (self.radius, self.length, self.n_y, self.n_z, self.pixel, self.sigma_z,
                self.sigma_dl)


WORKLOADS = {
    # 5 mm plain CPU-runnable case: 200 x 180, 1e6 events, 3-ellipse phantom, 10 iterations
    "plain-5mm-1M": Workload("plain-5mm-1M", 450.0, 1000.0, 180, 200, 5.0, 10.0, 42.0,
                             1_000_000, 10, 1, "three"),
    # full-size plain GPU case: 500 x 450 at 2 mm, 2e7 events, 10 ellipses, 20 iterations
    "plain-2mm-20M": Workload("plain-2mm-20M", 450.0, 1000.0, 450, 500, 2.0, 10.0, 42.0,
                              20_000_000, 20, 2, "random10"),
    # precision stress: 1000 x 900 at 1 mm, sigma 5 / 20, lesions at 8x, 1e8 events
    "stress-1mm-100M": Workload("stress-1mm-100M", 450.0, 1000.0, 900, 1000, 1.0, 5.0, 20.0,
                                100_000_000, 30, 5, "lesions"),
}
