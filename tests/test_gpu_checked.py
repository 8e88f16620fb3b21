"""The LK kernels' bounds, confirmed by the checked build (libvtg_checked.so, -DVTG_CHECKED): every template build,
window pass and sample pass tests its pixel rectangle against its level before reading. The workloads below (odd
sizes, the smallest and largest patches, points on and past the borders with guesses up to 150 px, a batched step)
must trip no test, and must give the same bits as the production build, which has no tests."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKLOAD = r"""
import ctypes as C, json, sys
sys.path[:0] = [%(pkg)r, %(oracle)r]
import numpy as np
import vtg, vtg_synth as S, oracle as O

ctx = vtg.Context(0)
out = {}
cases = [(640, 480, 3, 21, 21), (1281, 719, 5, 29, 31), (97, 61, 4, 7, 5), (1920, 1080, 4, 21, 21), (48, 40, 2, 5, 5)]
for k, (w, h, levels, pw, ph) in enumerate(cases):
    f0, f1, _, _ = S.warp_pair(w, h, S.seeded_shift(80 + k, 0), 0.5, seed=80 + k)
    t = vtg.Tracker(ctx, vtg.config(w, h, levels=levels, patch_w=pw, patch_h=ph, cell_w=8, cell_h=8))
    t.build(0, f0)
    t.build(1, f1)
    cells, lk = t.cells(0, 1)
    u = S.uniform(80 + k, 9, 4 * 256).reshape(4, 256)
    xs = (-5 + u[0] * (w + 10)).astype(np.float32)
    ys = (-5 + u[1] * (h + 10)).astype(np.float32)
    gx = (-150 + 300 * u[2]).astype(np.float32)
    gy = (-150 + 300 * u[3]).astype(np.float32)
    pts = t.points(0, 1, xs, ys, gx, gy)
    pts0 = t.points(1, 0, xs, ys)
    out["case%%d" %% k] = [O.fnv(cells), O.fnv(lk), O.fnv(pts), O.fnv(pts0)]
    t.close()
# a batched step over three of them
import torch
sizes = [(640, 480), (352, 288), (1280, 720)]
trs = [vtg.Tracker(ctx, vtg.config(w, h, levels=4)) for w, h in sizes]
pairs = [S.warp_pair(w, h, S.seeded_shift(90 + i, 0), 0.5, seed=90 + i)[:2] for i, (w, h) in enumerate(sizes)]
dev = [(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()) for a, b in pairs]
torch.cuda.synchronize()
for t, (a, _) in zip(trs, dev):
    t.build(0, a.data_ptr(), where=vtg.DEVICE)
ctx.sync()
b = vtg.Batch(ctx, 4)
b.prepare(0, trs, [d1.data_ptr() for _, d1 in dev], [1] * 3)
b.launch(0)
ctx.sync()
out["batch"] = [O.fnv(np.concatenate([x.view(np.uint8) for x in vtg.tracker_results(t)])) for t in trs]
word = (C.c_uint32 * 2)()
out["checked"] = vtg.lib().vtg_check_read(word)
out["word"] = [word[0], word[1]]
print(json.dumps(out))
"""


def _run(lib=None):
    env = dict(os.environ)
    if lib:
        env["VTG_LIB"] = lib
    else:
        env.pop("VTG_LIB", None)
    code = WORKLOAD % {"pkg": os.path.join(ROOT, "intel-phi-visiontrack_gb300"), "oracle": os.path.join(ROOT, "oracle")}
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_lk_windows_stay_inside_their_levels(vtg_lib):
    import vtg_build

    checked = _run(vtg_build.build(checked=True))
    assert checked["checked"] == 1, "the checked build did not load"
    assert checked["word"] == [0, 0], "a patch operation's rectangle left its level: sites %#x, %d times" % tuple(
        checked["word"])
    plain = _run()
    assert plain["checked"] == 0
    assert {k: v for k, v in checked.items() if k not in ("checked", "word")} == \
        {k: v for k, v in plain.items() if k not in ("checked", "word")}
