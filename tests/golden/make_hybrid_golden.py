"""Regenerates hybrid_ref.npz: outputs of the reference's own 3D hybrid
reconstruction (PET3D::Hybrid::Reconstruction<Scanner, GaussianKernel<float>>,
src/3d/hybrid/reconstruction.h), compiled from the reference headers by
oracle/build_ref.sh into oracle/_ref/ref_hybrid (one thread, no FP contraction),
on the small synthetic ring of the "hybrid-tiny" configuration.  The reference
has no test of this reconstruction, so these runs are what pins the CPU
restatement (oracle/hybrid_oracle.inc) and, through it, the GPU path.

Four cases, each stored with its inputs (geometry arrays, responses) so that
the test does not depend on the generator's floating point on another host:
  computed    weights from calculate_weight, sensitivity from
              calculate_sensitivity (the command without --system / --sensitivity)
  given       seeded system-matrix weights and --sens-to-one
  multiplane  one seeded system matrix per plane half (n_planes / 2 of them) and
              the 3D sensitivity from calculate_sensitivity
  sens3d      seeded system-matrix weights and a seeded external 3D sensitivity
              (--sensitivity, n_planes / 2 planes)
The last two read, for a voxel of plane iz, the weight and sensitivity plane
|iz - n_planes / 2|, which for plane 0 is one plane past the reference's arrays
(reconstruction.h:343-357); their responses are therefore those whose frame
event starts at plane 1 or later.
Outputs per case: the kept frame events, the normalized weights, the
sensitivity, rho after each of the iterations and the reference's statistics.

usage: python tests/golden/make_hybrid_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "j-pet-mlem_gb300", "python"))
from jpet_strip import hybrid_workloads as H  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_hybrid")


def write_case(path, g, resp, weights_given, sens_to_one, n_iter, sens_3d=None):
    h = g.n_planes_half
    with open(path, "w") as f:
        f.write(f"{g.n_detectors} {g.n_pixel_infos} {g.n_columns} {g.n_rows} {g.n_planes}\n")
        f.write(" ".join(f"{float(v):.9g}" for v in (
            g.pixel_size, g.lower_left_x, g.lower_left_y, g.z_left, g.sigma_z, g.sigma_dl,
            g.length)) + "\n")
        f.write(f"{int(weights_given)} {int(sens_to_one)} {n_iter} {h} "
                f"{int(sens_3d is not None)}\n")
        for l in range(g.n_lors):
            s = g.segments[l]
            f.write(" ".join(f"{float(s[n]):.9g}" for n in H.SEGMENT_DTYPE.names))
            f.write(f" {float(g.widths[l]):.9g} {int(g.info_begin[l])} {int(g.info_end[l])}\n")
        n = g.n_pixel_infos
        for i in range(n):
            f.write(f"{int(g.pixels[i]['x'])} {int(g.pixels[i]['y'])} "
                    f"{float(g.positions[i]):.9g} " +
                    " ".join(f"{float(g.weights[i + n * k]):.9g}" for k in range(h)) + "\n")
        if sens_3d is not None:
            f.write(" ".join(f"{float(v):.9g}" for v in sens_3d) + "\n")
        f.write(f"{resp.shape[0]}\n")
        for r in resp:
            f.write(f"{int(r['first'])} {int(r['second'])} {float(r['z_up']):.9g} "
                    f"{float(r['z_dn']):.9g} {float(r['dl']):.9g}\n")


def read_out(path, g, n_iter, depth=1):
    raw = open(path, "rb").read()
    off = 0
    n = int(np.frombuffer(raw, np.int64, 1, off)[0])
    off += 8
    packed = np.dtype([("first", "<i2"), ("second", "<i2"), ("up", "<f4"), ("right", "<f4"),
                       ("tan", "<f4"), ("sec", "<f4"), ("info_begin", "<u8"),
                       ("info_end", "<u8"), ("plane_begin", "<i2"), ("plane_end", "<i2")])
    ev = np.frombuffer(raw, packed, n, off)
    off += n * packed.itemsize
    frame = np.zeros(n, H.FRAME_EVENT_DTYPE)
    for name in packed.names:
        frame[name] = ev[name]
    nw = g.n_pixel_infos * g.n_planes_half
    w = np.frombuffer(raw, np.float32, nw, off).copy()
    off += 4 * nw
    ns = depth * g.n_columns * g.n_rows
    sens = np.frombuffer(raw, np.float32, ns, off).copy()
    off += 4 * ns
    rhos, stats = [], []
    for _ in range(n_iter):
        rhos.append(np.frombuffer(raw, np.float32, g.n_voxels, off).copy())
        off += 4 * g.n_voxels
        stats.append(np.frombuffer(raw, np.int64, 3, off).copy())
        off += 24
    assert off == len(raw)
    return frame, w, sens, np.stack(rhos), np.stack(stats)


def run_case(g, resp, weights_given, sens_to_one, n_iter, sens_3d=None):
    depth = (g.n_planes_half if g.n_planes_half > 1
             else (g.n_planes // 2 if sens_3d is not None else 1))
    with tempfile.TemporaryDirectory() as d:
        case, out = os.path.join(d, "case.txt"), os.path.join(d, "out.bin")
        write_case(case, g, resp, weights_given, sens_to_one, n_iter, sens_3d)
        subprocess.run([HARNESS, case, out], check=True)
        return read_out(out, g, n_iter, depth)


def from_plane_one(g, resp, weights):
    """The responses whose frame event (translated by the oracle, which is bit
    for bit the reference's) starts at plane 1 or later."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    keep = []
    for r in resp:
        fr = oracle.hybrid_translate(g, weights, r[None])
        if fr.shape[0] == 0 or int(fr["plane_begin"][0]) >= 1:
            keep.append(r)
    return np.array(keep, H.RESPONSE_DTYPE)


def edge_responses(g, seed):
    """Responses at the edges the reference handles: axial positions past the
    grid on either side (dropped by the bounding-box filter), at its ends (plane
    range clamped), and along-LOR positions near both detectors (info range at
    the LOR's first pixel info and one past its last)."""
    rng = np.random.default_rng(seed)
    out = np.zeros(40, H.RESPONSE_DTYPE)
    lors = rng.integers(1, g.n_detectors - 1, (40, 2))
    out["first"] = np.maximum(lors[:, 0], lors[:, 1] - 1) + 1
    out["second"] = np.minimum(lors[:, 0], lors[:, 1] - 1)
    half = float(g.n_planes) * g.pixel_size / 2
    z = np.concatenate([np.full(8, 2.5 * half), np.full(8, -2.5 * half),
                        rng.choice([-1.0, 1.0], 8) * (half - 0.3 * g.pixel_size),
                        rng.uniform(-0.5, 0.5, 16) * half])
    f = out["first"].astype(np.int64)
    R = g.segments["length"][f * (f + 1) // 2 + out["second"]] / 2
    dl = np.concatenate([rng.normal(0, g.sigma_dl, 24),
                         rng.choice([-1.0, 1.0], 16) * 2 * R[24:] * 0.95])
    out["z_up"] = z
    out["z_dn"] = z
    out["dl"] = dl
    return out


def main():
    data = {}
    cases = (("computed", "computed", False, 1, False), ("given", "given", True, 1, False),
             ("multiplane", "given", False, 6, False), ("sens3d", "given", False, 1, True))
    for tag, weights, sens_to_one, h, s3 in cases:
        g, n, n_iter = H.workload("hybrid-tiny", weights=weights)
        seed = {"computed": 5, "given": 6, "multiplane": 7, "sens3d": 8}[tag]
        if h > 1:
            g = H.multiplane_weights(g, h, seed=seed)
        resp = np.concatenate([H.responses(g, n, seed=seed), edge_responses(g, seed)])
        sens_in = None
        if s3:
            sens_in = np.random.default_rng(seed).uniform(
                0.5, 1.5, (g.n_planes // 2) * g.n_columns * g.n_rows).astype(np.float32)
        if h > 1 or s3:
            resp = from_plane_one(g, resp, g.weights)
        frame, w, sens, rhos, stats = run_case(g, resp, weights == "given", sens_to_one, n_iter,
                                               sens_in)
        for k, v in dict(segments=g.segments, widths=g.widths, pixels=g.pixels,
                         positions=g.positions, weights_in=g.weights, info_begin=g.info_begin,
                         info_end=g.info_end, responses=resp, frame=frame, weights=w, sens=sens,
                         rho=rhos, stats=stats).items():
            data[f"{tag}_{k}"] = v
        if sens_in is not None:
            data[f"{tag}_sens_in"] = sens_in
        data[f"{tag}_grid"] = np.array([g.n_detectors, g.n_columns, g.n_rows, g.n_planes,
                                        int(weights == "given"), int(sens_to_one), n_iter,
                                        h, int(s3)], np.int64)
        data[f"{tag}_params"] = np.array([g.pixel_size, g.lower_left_x, g.lower_left_y, g.z_left,
                                          g.sigma_z, g.sigma_dl, g.length, g.radius],
                                         np.float64)
        print(tag, "events kept", frame.shape[0], "of", resp.shape[0], "stats", stats[-1])
    np.savez_compressed(os.path.join(HERE, "hybrid_ref.npz"), **data)
    print("wrote hybrid_ref.npz")


if __name__ == "__main__":
    main()
