"""The drop-in, shown on the reference's own callers: its unmodified programs compiled with their _vx pyramid and LK
kernels redirected to this library's reference-signature entry points (include/vtg_compat.h) and linked against
libvtg.so, by oracle/Makefile's `dropin` target from the reference's sources (the tree where it exists, else the copy
in baseline/_ref that build() makes).

  - m2_ref 640 480 (src/host/m2_ref.c:44-78): its ten exact displacements x 330 points, every pyramid row and every
    LK track computed on the GPU. A shim beside each call runs the reference's own _vx kernel on the same arguments:
    every pyramid row is the same bits, and every track both call good is within 0.01 px of the host lane model, with
    at least 99 % of statuses equal. Its printed lk_first records agree with the CPU program's.
  - vt_replay translate 640x480 --mono --gate (src/host/vt_replay.c:125-264): the whole tracker (tk_build's pyramid
    and tk_track's feature LK with flowback on the GPU, everything else the reference's own C) held to the scene's own
    gate, tests/scenes.md:13 of the reference (continuity >= 0.99, EPE median <= 0.02 px, centre median <= 0.05 px),
    and its EPE within 0.005 px of the CPU replay's."""
import os
import re
import struct
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
DROPIN = os.path.join(ORACLE, "_ref", "dropin")


@pytest.fixture(scope="module")
def programs(vtg_lib):
    r = subprocess.run(["make", "-s", "-j8", "-C", ORACLE, "dropin"], capture_output=True, text=True)
    if r.returncode != 0 or not os.path.exists(os.path.join(DROPIN, "vt_replay_cuda")):
        pytest.skip("the reference's sources are not on this host (no tree, no baseline/_ref copy): " + r.stderr[-300:])
    return DROPIN


def _float(hexbits):
    return struct.unpack("<f", struct.pack("<I", int(hexbits, 16)))[0]


def _firsts(text):
    out = {}
    for m in re.finditer(r"lk_first (\S+) x ([0-9a-f]+) y ([0-9a-f]+) .* st (\d+)", text):
        out[m.group(1)] = (_float(m.group(2)), _float(m.group(3)), int(m.group(4)))
    return out


def test_m2_ref_on_the_gpu(programs):
    gpu = subprocess.run([os.path.join(programs, "m2_ref_cuda"), "640", "480"], capture_output=True, text=True,
                         timeout=600)
    assert gpu.returncode == 0, gpu.stderr[-2000:]
    m = re.search(r"dropin rows (\d+) rows_differ (\d+) points (\d+) both_ok (\d+) status_agree (\d+) "
                  r"max_err_px ([0-9.eE+-]+) compat_errors (\d+)", gpu.stderr)
    assert m, gpu.stderr[-2000:]
    rows, differ, points, both_ok, agree = (int(m.group(i)) for i in (1, 2, 3, 4, 5))
    err, cerr = float(m.group(6)), int(m.group(7))
    assert cerr == 0
    assert rows > 0 and differ == 0  # the pyramid is the reference's, bit for bit
    assert points == 10 * 330 and agree >= 0.99 * points and both_ok > 0.9 * points
    assert err <= 0.01
    cpu = subprocess.run([os.path.join(programs, "m2_ref"), "640", "480"], capture_output=True, text=True, timeout=600)
    assert cpu.returncode == 0
    g, c = _firsts(gpu.stdout), _firsts(cpu.stdout)
    assert len(g) == len(c) == 10
    for k in c:
        assert g[k][2] == c[k][2]
        if c[k][2] == 0:
            assert abs(g[k][0] - c[k][0]) <= 0.01 and abs(g[k][1] - c[k][1]) <= 0.01, (k, g[k], c[k])


def _score(path):
    """The figures the test reads from the replay's score file (src/host/score.c writes it as JSON-like fragments,
    not one JSON document, so they are read by name)."""
    text = open(path).read()
    num = r"(-?[0-9.]+)"
    epe = re.search(r'"epe_px":\{"n":(\d+),"median":' + num, text)
    return {"continuity": float(re.search(r'"continuity":' + num, text).group(1)),
            "epe_n": int(epe.group(1)), "epe_median": float(epe.group(2)),
            "id_changes": int(re.search(r'"id_changes":(\d+)', text).group(1)),
            "hidden_said_observed": int(re.search(r'"hidden_said_observed":(\d+)', text).group(1))}


def _replay(prog, tmp, name):
    out = os.path.join(tmp, name + ".json")
    r = subprocess.run([prog, "translate", "640x480", "--mono", "--gate", "--frames", "60", "--json", out], cwd=tmp,
                       capture_output=True, text=True, timeout=900)
    return r, _score(out) if os.path.exists(out) else None


def test_vt_replay_tracker_on_the_gpu_passes_the_scene_gate(programs, tmp_path):
    tmp = str(tmp_path)
    gpu, gs = _replay(os.path.join(programs, "vt_replay_cuda"), tmp, "gpu")
    assert gpu.returncode == 0, "the scene gate: " + gpu.stderr[-3000:]
    assert "GATE MISS" not in gpu.stderr
    cpu, cs = _replay(os.path.join(programs, "vt_replay"), tmp, "cpu")
    assert cpu.returncode == 0, cpu.stderr[-2000:]
    assert gs["continuity"] >= 0.99 and gs["epe_median"] <= 0.02
    assert gs["epe_n"] > 0.9 * cs["epe_n"]
    assert abs(gs["epe_median"] - cs["epe_median"]) <= 0.005
    assert gs["id_changes"] == 0 and gs["hidden_said_observed"] == 0
