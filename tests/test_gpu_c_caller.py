"""The C ABI from a C program (tests/c/track_pair.c): two frames of an analytic pattern moved by a known sub-pixel
shift, pyramids and per-cell flow through vtg.h from C. The median flow is the shift."""
import json
import subprocess

import pytest

from test_abi import _build_c_caller

pytestmark = pytest.mark.gpu


def test_c_program_tracks_a_known_shift(vtg_lib, tmp_path):
    exe = _build_c_caller(vtg_lib, tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["cells"] == 80 * 90 and out["good"] > 0.9 * out["cells"]
    assert abs(out["median_u"] - out["dx"]) < 0.02 and abs(out["median_v"] - out["dy"]) < 0.02, out
