"""The host command-line tool 2d_strip_reconstruction: the reference's options,
input formats and output naming (src/2d/strip/reconstruction_cmd.cpp:105-301)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOOL = os.path.join(ROOT, "j-pet-mlem_gb300", "bin", "2d_strip_reconstruction")

pytestmark = pytest.mark.skipif(not os.path.exists(TOOL), reason="host tool not built")

GEOM = ["-r", "450", "-l", "1000", "-p", "5", "--n-z-pixels", "200", "--n-y-pixels", "180",
        "--s-z", "10", "--s-dl", "42"]


def run(args, cwd=None):
    return subprocess.run([TOOL] + args, capture_output=True, text=True, cwd=cwd, timeout=300)


def test_usage_without_arguments():
    r = run([])
    assert r.returncode == 0
    for opt in ["--radius", "--length", "--s-pixel", "--n-z-pixels", "--n-y-pixels", "--s-z",
                "--s-dl", "--blocks", "--iterations", "--output", "--gpu", "--cuda-device",
                "--rho", "--rho-is-int", "--3d-response", "--dl-is-time", "--scale-length"]:
        assert opt in r.stderr


def test_missing_input_and_bad_option():
    r = run(["-i", "1"])
    assert r.returncode == 1 and "at least one responses input file expected" in r.stderr
    r = run(["--no-such-option", "x.bin"])
    assert r.returncode == 1 and "undefined option" in r.stderr
    r = run(["-i", "abc", "x.bin"])
    assert r.returncode == 1 and "option value is invalid" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("extra", [[], ["--precision", "1"], ["--kernel", "2"]])
def test_binary_input_matches_reference_golden(tmp_path, golden, extra):
    manifest, load = golden
    ev = load("c1_events.npy")
    ev.tofile(tmp_path / "ev.bin")
    r = run([str(tmp_path / "ev.bin")] + GEOM + ["-i", "3", "-I", "1", "-o",
                                                 str(tmp_path / "r.bin")] + extra)
    assert r.returncode == 0, r.stderr
    for it in (1, 3):
        got = np.fromfile(tmp_path / f"r_{it}.bin", np.float32).reshape(180, 200)
        want = load(f"c1_strict_it{it:02d}.npy")
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5
        nrrd = (tmp_path / f"r_{it}.nrrd").read_text()
        assert "sizes: 200 180" in nrrd and f"data file: ./r_{it}.bin" in nrrd


@pytest.mark.gpu
def test_text_input_and_tuples_output(tmp_path, golden):
    import oracle as O

    manifest, load = golden
    ev = load("c1_events.npy")[:3000]
    with open(tmp_path / "ev.txt", "w") as f:
        for zu, zd, dl in ev:
            f.write(f"{zu:.6f} {zd:.6f} {dl:.6f}\n")
    r = run([str(tmp_path / "ev.txt")] + GEOM + ["-i", "1", "-I", "2", "-o",
                                                 str(tmp_path / "t.txt")])
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "t_2.txt").read_text().split("\n")
    got = np.zeros((180, 200), np.float64)
    for ln in lines:
        if ln.strip():
            x, y, v = ln.split()
            got[int(y), int(x)] = float(v)
    parsed = np.loadtxt(tmp_path / "ev.txt", dtype=np.float64).astype(np.float32)
    want, _ = O.mlem_f(O.Geometry(450, 1000, 180, 200, 5, 10, 42), parsed, 2, threads=4)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5


@pytest.mark.gpu
def test_gpu_mode_output_protocol(tmp_path, golden):
    manifest, load = golden
    ev = load("c1_events.npy")[:2000]
    ev.tofile(tmp_path / "ev.bin")
    r = run([str(tmp_path / "ev.bin")] + GEOM + ["-i", "2", "-I", "3", "--gpu", "-v", "-o",
                                                 str(tmp_path / "g.bin")])
    assert r.returncode == 0, r.stderr
    names = sorted(p.name for p in tmp_path.iterdir() if p.suffix == ".bin" and p.name != "ev.bin")
    # sensitivity, iterations 1..3 of block 0 (i < I-1 and the block end), block end 6
    assert names == ["g_1.bin", "g_2.bin", "g_3.bin", "g_6.bin", "g_sensitivity.bin"]
    assert "# device:" in r.stderr


PHANTOM_TOOL = os.path.join(ROOT, "j-pet-mlem_gb300", "bin", "2d_strip_phantom")


def run_phantom(args, cwd=None):
    return subprocess.run([PHANTOM_TOOL] + args, capture_output=True, text=True, cwd=cwd,
                          timeout=300)


def test_phantom_tool_usage_and_errors(tmp_path):
    r = run_phantom([])
    assert r.returncode == 0
    for opt in ["--n-emissions", "--additive", "--detected", "--point", "--scale", "--output",
                "--image-origin", "--seed"]:
        assert opt in r.stderr
    r = run_phantom(["-r", "450", "-l", "1000", "-p", "5", "-e", "10"])
    assert r.returncode == 1 and "at least one input phantom description expected" in r.stderr
    (tmp_path / "bad.txt").write_text("hexagon 0 0 1 1 1\n")
    r = run_phantom(["-r", "450", "-l", "1000", "-p", "5", "-e", "10", str(tmp_path / "bad.txt")])
    assert r.returncode == 1 and "unknown phantom type: hexagon" in r.stderr
    golden = os.path.join(ROOT, "tests", "golden", "phantom_three.txt")
    r = run_phantom(["-r", "450", "-l", "1000", "-p", "5", "-e", "10", "--tan-bins", "-2",
                     golden])
    assert r.returncode == 1 and "--tan-bins must not be negative" in r.stderr
    r = run_phantom(["-r", "450", "-l", "1000", "-p", "5", "-e", "10", "--tan-bins", "4",
                     "--kernel-point", "1,2,3", golden])
    assert r.returncode == 1 and "--kernel-point must supply exactly 2 values" in r.stderr


@pytest.mark.gpu
def test_phantom_then_reconstruction_tool_chain(tmp_path):
    """2d_strip_phantom writes events, .cfg and count images; the reconstruction
    tool reads the events and loads the scanner options from the .cfg."""
    golden = os.path.join(ROOT, "tests", "golden", "phantom_three.txt")
    r = run_phantom(["-r", "450", "-l", "1000", "-p", "5", "--n-z-pixels", "200",
                     "--n-y-pixels", "180", "--s-z", "10", "--s-dl", "42", "-e", "200000",
                     "--seed", "7", "-o", str(tmp_path / "ph.bin"), golden])
    assert r.returncode == 0, r.stderr
    ev = np.fromfile(tmp_path / "ph.bin", np.float32).reshape(-1, 3)
    det = np.fromfile(tmp_path / "ph_detected", np.int32).reshape(180, 200)
    emi = np.fromfile(tmp_path / "ph_emitted", np.int32).reshape(180, 200)
    naive = np.fromfile(tmp_path / "ph_naive", np.int32).reshape(180, 200)
    assert 0.40 < len(ev) / 200000 < 0.44  # the reference detects ~0.420 of the emissions
    assert det.sum() == len(ev) and emi.sum() == 200000 and 0.9 * len(ev) < naive.sum() <= len(ev)
    cfg = (tmp_path / "ph.cfg").read_text()
    assert "--radius=450" in cfg and "--s-dl=42" in cfg and "--n-emissions=200000" in cfg
    assert "sizes: 200 180" in (tmp_path / "ph_detected.nrrd").read_text()
    # same seed, same stream; the text output holds the same events
    r = run_phantom(["-r", "450", "-l", "1000", "-p", "5", "--n-z-pixels", "200",
                     "--n-y-pixels", "180", "--s-z", "10", "--s-dl", "42", "-e", "200000",
                     "--seed", "7", "-o", str(tmp_path / "ph2.txt"), golden])
    assert r.returncode == 0, r.stderr
    ev2 = np.loadtxt(tmp_path / "ph2.txt", dtype=np.float32).reshape(-1, 3)
    assert ev2.shape == ev.shape and np.allclose(ev2, ev, rtol=1e-5, atol=1e-3)
    # --full: exact responses and emission events beside the smeared responses
    r = run_phantom(["-r", "450", "-l", "1000", "-p", "5", "--n-z-pixels", "200",
                     "--n-y-pixels", "180", "--s-z", "10", "--s-dl", "42", "-e", "20000",
                     "--seed", "7", "--full", "-o", str(tmp_path / "fu.bin"), golden])
    assert r.returncode == 0, r.stderr
    sm = np.fromfile(tmp_path / "fu.bin", np.float32).reshape(-1, 3)
    ex = np.fromfile(tmp_path / "fu_wo_error.bin", np.float32).reshape(-1, 3)
    fr = np.fromfile(tmp_path / "fu_full_response.bin", np.float32).reshape(-1, 3)
    evs = np.fromfile(tmp_path / "fu_events.bin", np.float32).reshape(-1, 4)
    assert len(sm) == len(ex) == len(fr) == len(evs) > 0 and np.array_equal(ex, fr)
    assert np.all(np.abs(ex[:, :2]) < 500.0)
    assert abs(float(np.std(sm[:, 0] - ex[:, 0])) - 10.0) < 0.5
    assert np.allclose(np.hypot(evs[:, 2], evs[:, 3]), 1.0, atol=1e-6)
    # --no-responses: images and .cfg only
    r = run_phantom(["-r", "450", "-l", "1000", "-p", "5", "--n-z-pixels", "200",
                     "--n-y-pixels", "180", "--s-z", "10", "--s-dl", "42", "-e", "20000",
                     "--seed", "7", "--no-responses", "-o", str(tmp_path / "nr.bin"), golden])
    assert r.returncode == 0, r.stderr
    assert not (tmp_path / "nr.bin").exists() and (tmp_path / "nr_naive").exists()
    assert (tmp_path / "nr.cfg").exists()
    # --tan-bins: the tangent-binned naive map and the kernel map (3D NRRD)
    r = run_phantom(["-r", "450", "-l", "1000", "-p", "5", "--n-z-pixels", "200",
                     "--n-y-pixels", "180", "--s-z", "10", "--s-dl", "42", "-e", "200000",
                     "--seed", "7", "--tan-bins", "6", "--kernel-point", "20,-10", "--detected",
                     "-o", str(tmp_path / "pt.bin"), golden])
    assert r.returncode == 0, r.stderr
    tmap = np.fromfile(tmp_path / "pt_tan_bins", np.int32).reshape(6, 180, 200)
    kmap = np.fromfile(tmp_path / "pt_tan_kernel", np.float32).reshape(6, 180, 200)
    naive_t = np.fromfile(tmp_path / "pt_naive", np.int32).reshape(180, 200)
    assert 0 < tmap.sum() <= naive_t.sum() and (tmap.sum(0) <= naive_t).all()
    assert np.isfinite(kmap).all() and kmap.max() > 0
    hdr = (tmp_path / "pt_tan_kernel.nrrd").read_text()
    assert "type: float" in hdr and "dimension: 3" in hdr and "sizes: 200 180 6" in hdr
    assert "type: int" in (tmp_path / "pt_tan_bins.nrrd").read_text()
    # reconstruction with the options of the accompanying .cfg only
    r = run([str(tmp_path / "ph.bin"), "-i", "2", "-I", "1", "-o", str(tmp_path / "r.bin")])
    assert r.returncode == 0, r.stderr
    img = np.fromfile(tmp_path / "r_2.bin", np.float32).reshape(180, 200)
    assert abs(img.sum() - len(ev)) < 1e-3 * len(ev)
