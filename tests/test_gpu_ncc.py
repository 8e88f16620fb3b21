"""GPU parity for the appearance search (F32 map), through the C ABI.

Bar: the per-cell map's corners, the eight candidates and the found corner in half pixels are identical to the
reference's (index work); scores agree within 1e-5 with the reference (32 x 21 on a Q6 plane) and within 1e-4 with the
FP64 oracle (T x T templates); near-blank windows always score 0."""
import os

import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch

    return torch


def _dev(torch, a):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    torch.cuda.synchronize()
    return t


def test_reference_32x21_on_q6_plane(vtg_lib, ctx, golden, torch_cuda):
    g = np.load(os.path.join(golden, "ncc_32x21.npz"))
    n0 = S.noise_frame(640, 480, seed=9)
    plane = O.pyramid(n0, 1)[0]
    app, norm = O.cut_template(plane, 300, 200, 32, 21)
    dp = _dev(torch_cuda, plane)
    s = vtg_lib.Search(ctx, 640, 480, 64, 64)
    s.template(app, norm)
    got = s.correlate(dp.data_ptr(), 640, 480, 640, vtg_lib.PLANE_F32, g["cx"], g["cy"])
    assert np.abs(got - g["corr"]).max() < 1e-5
    for key, (x0, x1, y0, y1, step) in (("s1", (250, 360, 150, 260, 1)), ("s2", (1, 640, 1, 480, 2))):
        f, mv, mx, my = s.run(dp.data_ptr(), 640, 480, 640, vtg_lib.PLANE_F32, x0, x1, y0, y1, step, want_map=True)
        n = len(g[key + "_map_v"])
        assert f["cells"] == n
        assert np.array_equal(mx, g[key + "_map_x"]) and np.array_equal(my, g[key + "_map_y"])
        assert np.abs(mv - g[key + "_map_v"]).max() < 1e-5
        assert [f["hx"], f["hy"]] == list(g[key])
        assert abs(f["ncc"] - float(g[key + "_ncc"])) < 1e-5 and abs(f["second"] - float(g[key + "_second"])) < 1e-5
    s.close()


def test_tracker_level_search(vtg_lib, ctx, torch_cuda):
    """Searching a tracker's resident pyramid level in place (the reacquisition path of try_reacquire)."""
    f0 = S.noise_frame(640, 480, seed=13)
    t = vtg_lib.Tracker(ctx, vtg_lib.config(640, 480, levels=3))
    t.build(0, f0)
    t.sync()
    ptr, w, h, pitch = vtg_lib.level_device(t, 0, 1)
    L1 = O.pyramid(f0, 2)[1]
    app, norm = O.cut_template(L1, 100, 70, 32, 21)
    s = vtg_lib.Search(ctx, w, h)
    s.template(app, norm)
    f = s.run(ptr, w, h, pitch, vtg_lib.PLANE_F32, 1, w, 1, h, 1)
    ref, _, _, _ = O.search_slot(L1, app, norm, 1, w, 1, h, 1, mode=O.F64)
    assert (f["hx"], f["hy"]) == (ref["hx"], ref["hy"]) == (200, 140)
    assert abs(f["ncc"] - ref["ncc"]) < 1e-4 and abs(f["ox"] - ref["ox"]) < 1e-3 and abs(f["oy"] - ref["oy"]) < 1e-3
    s.close()
    t.close()


@pytest.mark.parametrize("size", [(32, 32), (48, 24), (64, 64)])
def test_txt_templates_against_fp64_oracle(vtg_lib, ctx, torch_cuda, size):
    tw, th = size
    frame = S.noise_frame(320, 240, seed=21)
    plane = frame.astype(np.float32)
    tpl, xs, ys, blank = S.ncc_templates(frame, max(tw, th), 3, seed=5, blank_share=0.34)
    dp = _dev(torch_cuda, frame)
    s = vtg_lib.Search(ctx, 320, 240)
    for k in range(3):
        patch = tpl[k][:th, :tw].astype(np.float32)
        app = (patch - np.float32(patch.mean(dtype=np.float64))).astype(np.float32)
        norm = float(np.sum(app.astype(np.float64) ** 2))
        s.template(app, norm)
        f, mv, mx, my = s.run(dp.data_ptr(), 320, 240, 320, vtg_lib.PLANE_U8, 1, 320, 1, 240, 1, want_map=True)
        ref, rv, rx, ry = O.search_slot(plane, app, norm, 1, 320, 1, 240, 1, mode=O.F64)
        n = f["cells"]
        assert np.abs(mv - rv[:n]).max() < 1e-4
        same = np.abs(mv - rv[:n]) < 1e-6  # where two corners of a cell are within rounding, either may win
        assert np.array_equal(mx[same], rx[:n][same]) and np.array_equal(my[same], ry[:n][same])
        assert (f["hx"], f["hy"]) == (ref["hx"], ref["hy"])
        assert abs(f["ncc"] - ref["ncc"]) < 1e-4
        if blank[k]:
            assert f["ncc"] < 0.5
        else:
            assert (f["hx"] // 2, f["hy"] // 2) == (xs[k], ys[k]) and f["ncc"] > 0.9
    s.close()


@pytest.mark.parametrize("tw,th,step,window,plane_type,size", [
    (32, 21, 1, (7, 250, 3, 131), "u8", (320, 240)),     # 16 x 9 cells: a half-filled last row of 2 x 2 blocks
    (32, 21, 2, (5, 283, 9, 190), "f32", (320, 240)),    # 18 x 12 cells: 4 x 4 blocks, two columns of the last one
    (24, 7, 2, (1, 320, 1, 240), "u8", (320, 240)),      # 19 x 15 cells
    (128, 128, 1, (1, 320, 1, 240), "u8", (320, 240)),   # the largest template: the most shared memory a block takes
    (128, 128, 2, (3, 320, 2, 240), "f32", (320, 240)),
    (8, 1, 1, (2, 301, 1, 200), "u8", (320, 240)),       # the smallest template
    (72, 72, 1, (1, 640, 1, 480), "u8", (640, 480)),     # over 64 x 64 and most of the plane: integral images
    (80, 64, 2, (3, 640, 5, 480), "f32", (640, 480)),
])
def test_map_blocks_against_fp64_oracle(vtg_lib, ctx, torch_cuda, tw, th, step, window, plane_type, size):
    """The F32 map at the reference's steps (1 and 2) scores 32 x 32 corners a CTA; windows whose cells fill its last
    blocks only in part, at both plane types, with the window sums from the staged window and (a template over 64 x 64
    searching most of the plane) from the integral images, against the FP64 oracle's map and search."""
    W, H = size
    frame = S.noise_frame(W, H, seed=31 + tw + step)
    plane = frame.astype(np.float32)
    rng = np.random.default_rng(tw * 7 + th + step)
    tx, ty = int(rng.integers(window[0], min(window[1], W - tw - 2) + 1)), int(rng.integers(window[2], min(window[3], H - th - 2) + 1))
    patch = plane[ty:ty + th, tx:tx + tw]
    app = (patch - np.float32(patch.mean(dtype=np.float64))).astype(np.float32)
    norm = float(np.sum(app.astype(np.float64) ** 2))
    dp = _dev(torch_cuda, frame if plane_type == "u8" else plane)
    pt = vtg_lib.PLANE_U8 if plane_type == "u8" else vtg_lib.PLANE_F32
    s = vtg_lib.Search(ctx, W, H)
    s.template(app, norm)
    f, mv, mx, my = s.run(dp.data_ptr(), W, H, W, pt, *window, step, want_map=True)
    ref, rv, rx, ry = O.search_slot(plane, app, norm, *window, step, mode=O.F64)
    n = f["cells"]
    assert n > 0
    assert np.abs(mv - rv[:n]).max() < 1e-4
    same = np.abs(mv - rv[:n]) < 1e-6  # where two corners of a cell are within rounding, either may win
    assert np.array_equal(mx[same], rx[:n][same]) and np.array_equal(my[same], ry[:n][same])
    assert (f["hx"], f["hy"]) == (ref["hx"], ref["hy"])
    assert abs(f["ncc"] - ref["ncc"]) < 1e-4 and abs(f["second"] - ref["second"]) < 1e-4
    on_grid = tx % step == max(window[0], 1) % step and ty % step == max(window[2], 1) % step
    if on_grid and tw * th >= 256:  # a short row of smooth noise has near twins elsewhere
        assert (f["hx"], f["hy"]) == (2 * tx, 2 * ty) and f["ncc"] > 0.999
    s.close()


def test_near_blank_windows_score_zero(vtg_lib, ctx, torch_cuda):
    """vt_ncc_check's property on the GPU: nearly blank windows never read 0.5 or more, none reads over 1, and the
    template itself reads 1."""
    rng = np.random.default_rng(7)
    app = rng.integers(6000, 10000, size=(21, 32)).astype(np.float32)
    app -= np.float32(app.sum(dtype=np.float64) / app.size)
    norm = float((app.astype(np.float64) ** 2).sum())
    s = vtg_lib.Search(ctx, 64, 48)
    s.template(app, norm)
    worst = -2.0
    planes = []
    for level in (16320, 12800, 640):
        for step in (0, 1, 2, 4, 8, 16, 32, 64):
            for _ in range(8):
                planes.append((level - (rng.integers(0, step + 1, size=(48, 64)) if step else
                                        np.zeros((48, 64), int))).astype(np.float32))
    for pl in planes:
        dp = _dev(torch_cuda, pl)
        v = s.correlate(dp.data_ptr(), 64, 48, 64, vtg_lib.PLANE_F32, [4, 10, 20], [4, 10, 20])
        worst = max(worst, float(v.max()))
        assert (v <= 1.0 + 1e-6).all()
    assert worst < 0.5
    pl = np.full((48, 64), 8000.0, np.float32)
    pl[4:25, 4:36] += app
    dp = _dev(torch_cuda, pl)
    assert s.correlate(dp.data_ptr(), 64, 48, 64, vtg_lib.PLANE_F32, [4], [4])[0] > 0.999
    s.close()


def test_search_errors(vtg_lib, ctx):
    lib = vtg_lib.lib()
    s = vtg_lib.Search(ctx, 64, 64, 32, 32)
    f = vtg_lib.Found()
    import ctypes as C

    # no template yet
    assert lib.vtg_search_run(s.h, C.c_void_p(1), 64, 64, 64, 0, 0, 64, 0, 64, 1, 0, C.byref(f), None, None, None, 0,
                              None) == vtg_lib.EINVAL
    app = np.zeros((8, 16), np.float32)
    assert lib.vtg_search_template(s.h, app.ctypes.data, 40, 8, C.c_float(1.0), 0, None) == vtg_lib.EINVAL  # > max
    assert lib.vtg_search_template(s.h, app.ctypes.data, 12, 8, C.c_float(1.0), 0, None) == vtg_lib.EINVAL  # % 8
    s.template(app, 0.0)
    # the tensor-core map reads 8-bit planes only
    assert lib.vtg_search_run(s.h, C.c_void_p(1), 64, 64, 64, 1, 0, 64, 0, 64, 1, 1, C.byref(f), None, None, None, 0,
                              None) == vtg_lib.EINVAL
    s.close()
