"""The host tool 3d_tool_convert against the reference's own converter
(src/3d/tool/convert_cmd.cpp): the committed outputs of the reference binary
(tests/golden/make_convert_golden.py) are reproduced byte for byte, for the
Warsaw hit format (detector assignment on one and two rings, Gaussian
smearing from std::mt19937_64, --only, automatic detector width) and the
T. Bednarski time format; plus the reference's option errors.  Host code only:
no GPU."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
TOOL = os.path.join(ROOT, "j-pet-mlem_gb300", "bin", "3d_tool_convert")

pytestmark = pytest.mark.skipif(not os.path.exists(TOOL), reason="host tool not built")

with open(os.path.join(GOLDEN, "convert_ref.json")) as f:
    CASES = json.load(f)


def run(args):
    return subprocess.run([TOOL] + args, capture_output=True, text=True, cwd=GOLDEN, timeout=120)


@pytest.mark.parametrize("case", sorted(CASES))
def test_output_matches_the_reference_converter(case):
    args, want = CASES[case]
    r = run(args)
    assert r.returncode == 0, r.stderr
    assert want.count("\n") > 10
    assert r.stdout == want


def test_converted_responses_feed_the_3d_response_reader():
    """The Warsaw output is the "d1 d2 z_u z_d dl" layout the reconstruction
    tool reads with --3d-response: detector pairs ordered d1 >= d2, finite
    values, |z| within the scintillator half length plus smearing."""
    args, want = CASES["warsaw"]
    rows = [line.split() for line in want.strip().split("\n")]
    assert all(len(r) == 5 for r in rows)
    for r in rows:
        d1, d2 = int(r[0]), int(r[1])
        assert 0 <= d2 <= d1 < 48
        assert abs(float(r[2])) < 0.25 + 0.1 and abs(float(r[3])) < 0.25 + 0.1


def test_usage_and_option_errors():
    r = run([])
    assert r.returncode == 0
    assert "--w-detector, --d-detector, --n-detectors" in r.stderr
    for opt in ["--radius", "--rotation", "--n-detectors", "--warsaw", "--tbednarski", "--only",
                "--relative-time", "--seed"]:
        assert opt in r.stderr
    r = run(["convert_warsaw_hits.txt"])
    assert r.returncode == 1 and "need to specify either" in r.stderr
    r = run(["-r", "0.43", "-d", "30", "-w", "0.007", "convert_warsaw_hits.txt"])
    assert r.returncode == 1 and "number of detectors must be multiple of 4" in r.stderr
    r = run(["-r", "0.43", "-d", "48", "-w", "0.007", "--rotation", "0.3",
             "convert_warsaw_hits.txt"])
    assert r.returncode == 1 and "broken symmetry" in r.stderr
    r = run(["-r", "0.5,0.43", "-d", "48", "-w", "0.007", "convert_warsaw_hits.txt"])
    assert r.returncode == 1 and "incrementing order" in r.stderr
    r = run(["-r", "0.43", "-d", "48", "-w", "0.007", "no_such_file.txt"])
    assert r.returncode == 1 and "cannot open input means file: no_such_file.txt" in r.stderr
