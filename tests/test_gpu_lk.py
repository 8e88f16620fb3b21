"""GPU parity for the pyramid and LK, through the C ABI.

Bar: the pyramid is bit-exact (the reference's F32 planes are exact integers); the cell record's `diff` is bit-exact;
flow agrees with the FP64 oracle within 0.01 px max-abs on every cell both call good, and status agrees on at least 99 %
of cells (a cell whose minimum eigenvalue or bounds test sits on a threshold may flip between arithmetics)."""
import os

import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu

TOL_PX = 0.01


def _flow_err(a, b):
    ok = (a["status"] == 0) & (b["status"] == 0)
    err = np.maximum(np.abs(a["x"] - b["x"]), np.abs(a["y"] - b["y"]))[ok]
    return ok, (float(err.max()) if err.size else 0.0)


def _tracker(vtg_lib, ctx, w, h, **kw):
    return vtg_lib.Tracker(ctx, vtg_lib.config(w, h, **kw))


@pytest.mark.parametrize("w,h,levels", [(32, 32, 1), (33, 47, 3), (97, 61, 4), (640, 480, 3), (1281, 719, 5),
                                        (1920, 1080, 4),
                                        # levels 0-3 are made in 128 x 64 blocks of level 0: block (1, 1) just inside
                                        # the frame (its staged bytes end on the last column and row), just not, and a
                                        # one-pixel sliver of a block
                                        (272, 135, 4), (271, 134, 4), (129, 65, 4)])
def test_pyramid_bit_exact(vtg_lib, ctx, w, h, levels):
    frame = S.noise_frame(w, h, seed=w + 3 * h)
    t = _tracker(vtg_lib, ctx, w, h, levels=levels)
    t.build(1, frame)
    ref = O.pyramid(frame, levels)
    for L in range(levels):
        assert np.array_equal(t.level(1, L), ref[L]), "level %d" % L
    t.close()


def test_pyramid_strided_and_device_input(vtg_lib, ctx):
    import torch

    w, h = 650, 301
    frame = S.noise_frame(w, h, seed=4)
    padded = np.zeros((h, 704), np.uint8)
    padded[:, :w] = frame
    t = _tracker(vtg_lib, ctx, w, h, levels=3)
    t.build(0, padded, stride=704)
    dev = torch.from_numpy(padded).cuda()
    torch.cuda.synchronize()
    t.build(1, dev.data_ptr(), stride=704, where=vtg_lib.DEVICE)
    ref = O.pyramid(frame, 3)
    for L in range(3):
        assert np.array_equal(t.level(0, L), ref[L]) and np.array_equal(t.level(1, L), ref[L])
    t.close()


def test_pyramid_1080p_matches_reference_hashes(vtg_lib, ctx, golden):
    g = np.load(os.path.join(golden, "lk_1080p.npz"))
    f0, f1, _, _ = S.warp_pair(1920, 1080, S.seeded_shift(2, 0), 0.5, seed=2)
    t = _tracker(vtg_lib, ctx, 1920, 1080, levels=4)
    t.build(0, f0)
    t.build(1, f1)
    assert [O.fnv(t.level(0, L)) for L in range(4)] == [int(v) for v in g["pyr0_fnv"]]
    assert [O.fnv(t.level(1, L)) for L in range(4)] == [int(v) for v in g["pyr1_fnv"]]
    t.close()


def test_cells_config1(vtg_lib, ctx, golden):
    """640 x 480, 1,200 cells on a 16 px grid, 21 x 21, 3 levels, <= 10 iterations, eps 0.01, flowback 0.5."""
    g = np.load(os.path.join(golden, "lk_640x480.npz"))
    f0, f1, _, _ = S.warp_pair(640, 480, (1.7, -0.8), 0.5, seed=1)
    t = _tracker(vtg_lib, ctx, 640, 480, levels=3, cell_w=16, cell_h=16)
    t.build(0, f0)
    t.build(1, f1)
    cells, lk = t.cells(0, 1)
    assert len(cells) == 1200
    P0, P1 = O.pyramid(f0, 3), O.pyramid(f1, 3)
    olk, ocells = O.cells(P0, P1, 2, O.lk_cfg(), 16, 16, max_fb=0.5, mode=O.F64, threads=8)
    ok, err = _flow_err(lk, olk)
    assert (lk["status"] == olk["status"]).mean() >= 0.99
    assert err <= TOL_PX, err
    ref = g["vx"].view(O.LK_OUT)  # the reference's own lk_track_vx + lk_flowback_vx
    ok2, err2 = _flow_err(lk, ref)
    assert (lk["status"] == ref["status"]).mean() >= 0.99 and err2 <= TOL_PX
    assert np.array_equal(cells["diff"], ocells["diff"])
    good = cells["state"] == 0
    assert np.allclose(cells["u"][good], lk["x"][good] - g["xs"][good], atol=0)
    assert np.abs(cells["sigma"] - ocells["sigma"])[good & (ocells["state"] == 0)].max() < 1e-4


def test_cells_config2_full_and_half(vtg_lib, ctx, golden):
    """1920 x 1080, 4 levels: 16,200 cells (16 x 8) at level 0 and 4,080 at level 1."""
    g = np.load(os.path.join(golden, "lk_1080p.npz"))
    f0, f1, _, _ = S.warp_pair(1920, 1080, S.seeded_shift(2, 0), 0.5, seed=2)
    P0, P1 = O.pyramid(f0, 4), O.pyramid(f1, 4)
    for flow_level, n, top, sel, ref in ((0, 16200, 3, g["sel"], g["vx"]), (1, 4080, 2, g["half_sel"], g["half_vx"])):
        t = _tracker(vtg_lib, ctx, 1920, 1080, levels=4, cell_w=16, cell_h=8, flow_level=flow_level)
        t.build(0, f0)
        t.build(1, f1)
        cells, lk = t.cells(0, 1)
        assert len(cells) == n
        olk, ocells = O.cells(P0[flow_level:], P1[flow_level:], top, O.lk_cfg(), 16, 8, max_fb=0.5, mode=O.F64,
                              threads=8)
        ok, err = _flow_err(lk, olk)
        assert (lk["status"] == olk["status"]).mean() >= 0.99
        assert err <= TOL_PX, (flow_level, err)
        assert np.array_equal(cells["diff"], ocells["diff"])
        r = ref.view(O.LK_OUT)
        _, err2 = _flow_err(lk[sel], r)
        assert err2 <= TOL_PX
        t.close()


def test_points_with_guesses_and_borders(vtg_lib, ctx):
    """The point list (OP_LK) with per-point guesses, points past every border, a flat band and two patch sizes."""
    w, h = 200, 150
    f0, f1, _, _ = S.warp_pair(w, h, (2.5, -1.5), 0.5, seed=11)
    f0[:, :40] = 128
    f1[:, :40] = 128
    xs = np.array([5, 11, 12, 13, 100, 187, 188, 189, 195, 30, 60, 150, 100.25, 99.75], np.float32)
    ys = np.array([75, 75, 75, 75, 5, 75, 75, 75, 75, 75, 140, 12, 70.5, 71.125], np.float32)
    gx = np.linspace(-3, 3, len(xs)).astype(np.float32)
    gy = np.linspace(2, -2, len(xs)).astype(np.float32)
    for (pw, ph, levels, fb) in ((21, 21, 3, 0.5), (15, 15, 1, 0.25), (9, 13, 2, 0.0), (29, 31, 2, 0.5)):
        t = _tracker(vtg_lib, ctx, w, h, levels=levels, patch_w=pw, patch_h=ph, fb_max=fb)
        t.build(0, f0)
        t.build(1, f1)
        out = t.points(0, 1, xs, ys, gx, gy)
        P0, P1 = O.pyramid(f0, levels), O.pyramid(f1, levels)
        ref = O.lk_points(P0, P1, levels - 1, O.lk_cfg(pw, ph), xs, ys, gx, gy, max_fb=fb, mode=O.F64)
        assert np.array_equal(out["status"], ref["status"]), (pw, ph)
        ok, err = _flow_err(out, ref)
        assert err <= TOL_PX
        assert np.array_equal(out["iters"][ok], ref["iters"][ok]) or np.abs(
            out["iters"].astype(int) - ref["iters"].astype(int)).max() <= 1
        t.close()


def test_still_vectors_config(vtg_lib, ctx, golden):
    """The reference's own per-cell flow settings (15 x 15, one level, 6 iterations, flowback 0.25, 16 x 8 cells)
    against its still_vectors output."""
    g = np.load(os.path.join(golden, "still_vectors.npz"))
    f0, f1, _, _ = S.warp_pair(640, 480, (0.6, -0.3), 0.3, seed=5)
    t = _tracker(vtg_lib, ctx, 640, 480, levels=1, patch_w=15, patch_h=15, max_iter=6, max_residual=16.0,
                 fb_max=0.25, cell_w=16, cell_h=8)
    t.build(0, f0)
    t.build(1, f1)
    cells, lk = t.cells(0, 1)
    ref = g["cells"].view(O.CELL)
    assert np.array_equal(cells["diff"], ref["diff"])
    assert (cells["state"] == ref["state"]).mean() >= 0.99
    ok = (cells["state"] == 0) & (ref["state"] == 0)
    assert np.maximum(np.abs(cells["u"] - ref["u"]), np.abs(cells["v"] - ref["v"]))[ok].max() <= TOL_PX
    t.close()


def test_m2_accuracy_against_exact_truth(vtg_lib, ctx, golden):
    """The reference's accuracy table against exact truth (docs/measurements.md:93-104; the M2 gate's ten quarter-pixel
    displacements of its pattern, 330 points, 21 x 21, eps 0.005, 4 levels) through vtg_points: as many points with
    status OK (within 3, where a point sits on a threshold), and EPE median / p95 / max within 0.002 / 0.003 / 0.005 px
    of the table's on every displacement the reference tracks in full. On the last one, where the reference loses 27
    tracks to the pattern's repeats, the points both call good agree with the FP64 oracle within 0.01 px."""
    import json

    from test_oracle import m2_case_stats, m2_points

    with open(os.path.join(golden, "m1_m2.json")) as f:
        table = json.load(f)["m2_accuracy"]
    xs, ys = m2_points()
    cfg = O.lk_cfg(21, 21, 10, 0.005, 0.1, 40.0)
    t = _tracker(vtg_lib, ctx, 640, 480, levels=4, eps=0.005, max_residual=40.0, fb_max=0.0)
    f0 = O.m2_render(640, 480, 2048, 2048)
    t.build(0, f0)
    P0 = O.pyramid(f0, 4)
    for row in table:
        dx, dy = int(round(4 * row["d"][0])), int(round(4 * row["d"][1]))
        f1 = O.m2_render(640, 480, 2048 - dx, 2048 - dy)
        t.build(1, f1)
        out = t.points(0, 1, xs, ys)
        n, med, p95, mx = m2_case_stats(out, xs, ys, dx, dy)
        assert abs(n - row["ok"]) <= 3, (row, n)
        if row["ok"] == len(xs):
            assert n == row["ok"]
            assert abs(med - row["median"]) <= 0.002 and abs(p95 - row["p95"]) <= 0.003, (row, med, p95)
            assert abs(mx - row["max"]) <= 0.005, (row, mx)
        else:
            ref = O.lk_points(P0, O.pyramid(f1, 4), 3, cfg, xs, ys, mode=O.F64)
            ok, err = _flow_err(out, ref)
            assert err <= TOL_PX and np.mean(out["status"] == ref["status"]) >= 0.99
    t.close()


def test_repeatable_and_set_order(vtg_lib, ctx):
    """Same inputs, same bits, run after run; and the sets are symmetric (build order does not matter)."""
    f0, f1, _, _ = S.warp_pair(320, 240, (1.0, 0.5), 0.5, seed=3)
    t = _tracker(vtg_lib, ctx, 320, 240, levels=3, cell_w=16, cell_h=16)
    t.build(0, f0)
    t.build(1, f1)
    a = t.cells(0, 1)
    b = t.cells(0, 1)
    t.build(1, f0)
    t.build(0, f1)
    c = t.cells(1, 0)
    for x, y in ((a, b), (a, c)):
        assert x[0].tobytes() == y[0].tobytes() and x[1].tobytes() == y[1].tobytes()
    t.close()


def test_concurrent_streams_same_bits(vtg_lib, ctx):
    """Four trackers working at once, each on its own CUDA stream with nothing between them, give the same bits as the
    same work one tracker after another (the GPU form of the reference's team-size invariance)."""
    sizes = [(640, 480), (333, 199), (1280, 720), (97, 61)]
    pairs = [S.warp_pair(w, h, S.seeded_shift(60 + k, 0), 0.5, seed=60 + k)[:2] for k, (w, h) in enumerate(sizes)]
    alone = []
    for (w, h), (f0, f1) in zip(sizes, pairs):
        t = _tracker(vtg_lib, ctx, w, h, levels=3, cell_w=8, cell_h=8)
        t.build(0, f0)
        t.build(1, f1)
        alone.append(t.cells(0, 1))
        t.close()
    ts = [_tracker(vtg_lib, ctx, w, h, levels=3, cell_w=8, cell_h=8) for (w, h) in sizes]
    outs = []
    for t, (f0, f1) in zip(ts, pairs):  # enqueue everything first, read afterwards
        t.build(0, f0)
        t.build(1, f1)
        n = t.cols * t.rows
        c = np.zeros(n, vtg_lib.CELL_DTYPE)
        lk = np.zeros(n, vtg_lib.LK_OUT_DTYPE)
        vtg_lib.check(vtg_lib.lib().vtg_cells(t.h, 0, 1, c.ctypes.data, lk.ctypes.data, vtg_lib.HOST, None), "cells")
        outs.append((c, lk))
    ctx.sync()
    for (c, lk), (c0, lk0) in zip(outs, alone):
        assert c.tobytes() == c0.tobytes() and lk.tobytes() == lk0.tobytes()
    for t in ts:
        t.close()


def test_largest_frame(vtg_lib, ctx):
    """The largest frame a tracker takes, 16384 x 16384 (6 levels, 2.1 M cells): every level bit-exact, the cell grid
    computed, and its cells at 512 sampled places, plus 512 points with guesses, within 0.01 px of the FP64 oracle.
    Offsets here pass 2^28 elements a plane, so any 32-bit index arithmetic would show."""
    w = h = 16384
    base = S.noise_frame(1024, 1024, seed=77)
    frame = np.tile(base, (16, 16))
    frame[::7, ::5] ^= 0x5A  # break the tiling's periodicity
    f1 = np.roll(frame, (3, -2), axis=(0, 1))
    t = _tracker(vtg_lib, ctx, w, h, levels=6)
    t.build(0, frame)
    t.build(1, f1)
    P0, P1 = O.pyramid(frame, 6), O.pyramid(f1, 6)
    for L in range(6):
        assert np.array_equal(t.level(1, L), P1[L]), "level %d" % L
    cells, lk = t.cells(0, 1)
    assert len(cells) == (w // 16) * (h // 8)
    cfg = O.lk_cfg()
    sel = np.sort(S.hash_u64(77, 1, 512) % len(cells)).astype(np.int64)
    xs, ys = O.cell_centres(w, h, 16, 8)
    ref = O.lk_points(P0, P1, 5, cfg, xs[sel], ys[sel], max_fb=0.5, mode=O.F64, threads=os.cpu_count() or 1)
    ok, err = _flow_err(lk[sel], ref)
    assert err <= TOL_PX and np.mean(lk[sel]["status"] == ref["status"]) >= 0.99
    u = S.uniform(77, 2, 4 * 512).reshape(4, 512)
    px = (20 + u[0] * (w - 40)).astype(np.float32)
    py = (20 + u[1] * (h - 40)).astype(np.float32)
    gx = (-3 + 6 * u[2]).astype(np.float32)
    gy = (-3 + 6 * u[3]).astype(np.float32)
    got = t.points(0, 1, px, py, gx, gy)
    ref = O.lk_points(P0, P1, 5, cfg, px, py, gx, gy, max_fb=0.5, mode=O.F64, threads=os.cpu_count() or 1)
    ok, err = _flow_err(got, ref)
    assert err <= TOL_PX and np.mean(got["status"] == ref["status"]) >= 0.99 and ok.mean() > 0.5
    t.close()


NONFINITE = r"""
import ctypes as C, json, sys
sys.path[:0] = [%(pkg)r, %(oracle)r]
import numpy as np
import vtg, vtg_synth as S
ctx = vtg.Context(0)
f0, f1, _, _ = S.warp_pair(320, 240, (1.2, -0.7), 0.4, seed=31)
t = vtg.Tracker(ctx, vtg.config(320, 240, levels=3))
t.build(0, f0)
t.build(1, f1)
nan, inf = float("nan"), float("inf")
xs = np.array([160, nan, 100, inf, -inf, 200, 120, 150, 1e30, 80], np.float32)
ys = np.array([120, 100, nan, 100, 100, inf, 90, 130, 100, 60], np.float32)
gx = np.array([0, 0, 0, 0, 0, 0, nan, inf, 0, -1e30], np.float32)
gy = np.array([0, 0, 0, 0, 0, 0, 0, 0, 0, 0], np.float32)
out = t.points(0, 1, xs, ys, gx, gy)
clean = t.points(0, 1, xs[:1], ys[:1], gx[:1], gy[:1])
word = (C.c_uint32 * 2)()
checked = vtg.lib().vtg_check_read(word)
print(json.dumps({"status": out["status"].tolist(), "first": out[:1].tobytes().hex(),
                  "clean": clean.tobytes().hex(), "checked": checked, "word": [word[0], word[1]]}))
"""


def test_points_with_nonfinite_inputs(vtg_lib):
    """Points and guesses that are NaN, infinite or absurd are VTG_LK_OUT, never a window read at a garbage place, and
    the good point beside them gets the same bits as alone. Run first through the bounds-checked build, whose window
    tests would record (and skip) any read outside a level, then through the production build."""
    import json
    import subprocess
    import sys

    import vtg_build

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = NONFINITE % {"pkg": os.path.join(root, "intel-phi-visiontrack_gb300"), "oracle": os.path.join(root, "oracle")}
    results = []
    for lib in (vtg_build.build(checked=True), None):
        env = dict(os.environ)
        env.pop("VTG_LIB", None)
        if lib:
            env["VTG_LIB"] = lib
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
        res = json.loads(r.stdout.strip().splitlines()[-1])
        if lib:
            assert res["checked"] == 1 and res["word"] == [0, 0], res["word"]
        results.append(res)
    for res in results:
        st = res["status"]
        assert st[0] == 0 and res["first"] == res["clean"]
        assert all(s & 1 for s in st[1:]), st  # VTG_LK_OUT
    assert results[0]["status"] == results[1]["status"]


def test_empty_point_list(vtg_lib, ctx):
    f0, f1, _, _ = S.warp_pair(64, 64, (1.0, 0.5), 0.5, seed=4)
    t = _tracker(vtg_lib, ctx, 64, 64, levels=2)
    t.build(0, f0)
    t.build(1, f1)
    out = t.points(0, 1, np.zeros(0, np.float32), np.zeros(0, np.float32))
    assert len(out) == 0
    t.close()


def test_errors_are_status_codes(vtg_lib, ctx):
    lib = vtg_lib.lib()
    t = _tracker(vtg_lib, ctx, 64, 64, levels=2)
    assert lib.vtg_build(t.h, 2, None, 64, 0, None) == vtg_lib.EINVAL
    assert lib.vtg_cells(t.h, 0, 3, None, None, 0, None) == vtg_lib.EINVAL
    assert lib.vtg_points(t.h, 0, 1, 5, 1, None, None, None, None, None, 0, None) == vtg_lib.EINVAL
    t.close()
    small = vtg_lib.Context(0, hbm_budget=1 << 20)
    with pytest.raises(vtg_lib.VtgError) as e:
        vtg_lib.Tracker(small, vtg_lib.config(1920, 1080))
    assert e.value.code == vtg_lib.EBUDGET
    small.close()


def test_points_two_warps_a_point(vtg_lib, ctx):
    """The point list walked by two warps a point, each over half the patch's rows (vtg_tracker_set_point_warps):
    the same points as one warp a point up to the F32 rounding of the sums, and within 0.01 px of the FP64 oracle, for
    patches whose halves are even, odd and unequal."""
    w, h = 320, 240
    f0, f1, _, _ = S.warp_pair(w, h, (1.5, -2.25), 0.5, seed=21)
    rng = np.random.default_rng(21)
    xs = rng.uniform(20, w - 20, 200).astype(np.float32)
    ys = rng.uniform(20, h - 20, 200).astype(np.float32)
    for (pw, ph, levels, fb) in ((21, 21, 3, 0.5), (15, 15, 2, 0.25), (9, 13, 2, 0.0), (29, 31, 2, 0.5)):
        t = _tracker(vtg_lib, ctx, w, h, levels=levels, patch_w=pw, patch_h=ph, fb_max=fb)
        t.build(0, f0)
        t.build(1, f1)
        t.set_point_warps(1)
        one = t.points(0, 1, xs, ys)
        t.set_point_warps(2)
        two = t.points(0, 1, xs, ys)
        t.set_point_warps(0)
        auto = t.points(0, 1, xs, ys)
        assert auto.tobytes() == one.tobytes()  # the default is one warp a point
        assert (one["status"] == two["status"]).mean() >= 0.99, (pw, ph)
        both = (one["status"] == 0) & (two["status"] == 0)
        assert both.sum() > 0.5 * len(xs)
        assert np.abs(one["x"] - two["x"])[both].max() <= 1e-3 and np.abs(one["y"] - two["y"])[both].max() <= 1e-3
        P0, P1 = O.pyramid(f0, levels), O.pyramid(f1, levels)
        ref = O.lk_points(P0, P1, levels - 1, O.lk_cfg(pw, ph), xs, ys, max_fb=fb, mode=O.F64)
        assert (two["status"] == ref["status"]).mean() >= 0.99
        ok, err = _flow_err(two, ref)
        assert err <= TOL_PX, (pw, ph, err)
        with pytest.raises(vtg_lib.VtgError):
            t.set_point_warps(3)
        t.close()
