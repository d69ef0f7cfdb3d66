"""Fits the arctangent polynomial of hybrid.cu (atan_poly): atan(r) = r P(r^2) on
r in [0, 1], P of degree 8, by iteratively reweighted least squares on
Chebyshev-spaced nodes (Lawson's algorithm towards the minimax fit of the
absolute error).  Prints the float32 coefficients and the error of the float32
Horner evaluation against numpy's double arctan.

usage: python j-pet-mlem_gb300/csrc/fit_atan.py
"""
import numpy as np

DEGREE = 8


def fit(deg: int = DEGREE, iterations: int = 30) -> np.ndarray:
    n = 4000
    s = (1 - np.cos(np.linspace(0, np.pi, n))) / 2
    r = np.sqrt(s)
    f = np.where(r > 0, np.arctan(r) / np.where(r > 0, r, 1), 1.0)
    w = np.ones(n)
    A = np.vander(s, deg + 1, increasing=True) * r[:, None]
    b = f * r
    for _ in range(iterations):
        c, *_ = np.linalg.lstsq(A * w[:, None], b * w, rcond=None)
        e = A @ c - b
        w = w * (np.abs(e) / np.abs(e).max() + 1e-3) ** 0.5
        w /= w.max()
    return c.astype(np.float32)


def horner_f32(c: np.ndarray, r: np.ndarray) -> np.ndarray:
    r = r.astype(np.float32)
    s = (r * r).astype(np.float32)
    p = np.float32(c[-1])
    for k in range(len(c) - 2, -1, -1):
        p = (p * s + c[k]).astype(np.float32)
    return (p * r).astype(np.float32)


def main():
    c = fit()
    r = np.linspace(0, 1, 2_000_001).astype(np.float32)
    err = np.abs(horner_f32(c, r).astype(np.float64) - np.arctan(r.astype(np.float64)))
    print("coefficients (c0 .. c8):")
    for v in c:
        print(f"  {float(v):.9e}f,")
    print(f"max |error| on [0, 1]: {err.max():.3e}")


if __name__ == "__main__":
    main()
