"""The tensor-core correlation map (tcgen05, BF16 / FP16 products, F32 accumulation) against the F32 map and the FP64
oracle. The map's values carry the products' rounding; the found corner and its score come from the F32 re-score of
the eight candidates, so they must agree with the F32 path's whenever the candidates do."""
import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu

TOL_MAP = {1: 0.02, 2: 0.005}  # BF16, FP16: max |map value - F32 map value|


def _dev(a):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    torch.cuda.synchronize()
    return t


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("tw,th,w,h", [(32, 21, 200, 100), (32, 32, 640, 480), (64, 64, 640, 480), (96, 96, 1100, 300),
                                      (128, 128, 640, 480), (128, 40, 700, 300)])
def test_tc_map_matches_f32_map(vtg_lib, ctx, precision, tw, th, w, h):
    frame = S.noise_frame(w, h, seed=tw + th + w)
    tpl, xs, ys, blank = S.ncc_templates(frame, max(tw, th), 2, seed=3, blank_share=0.0)
    patch = tpl[0][:th, :tw].astype(np.float32)
    app = (patch - np.float32(patch.mean(dtype=np.float64))).astype(np.float32)
    norm = float(np.sum(app.astype(np.float64) ** 2))
    dp = _dev(frame)
    s = vtg_lib.Search(ctx, w, h)
    s.template(app, norm)
    f32, v32, x32, y32 = s.run(dp.data_ptr(), w, h, w, vtg_lib.PLANE_U8, 1, w, 1, h, 1, vtg_lib.NCC_F32, want_map=True)
    ftc, vtc, xtc, ytc = s.run(dp.data_ptr(), w, h, w, vtg_lib.PLANE_U8, 1, w, 1, h, 1, precision, want_map=True)
    assert ftc["cells"] == f32["cells"]
    assert np.abs(vtc - v32).max() < TOL_MAP[precision]
    assert (ftc["hx"], ftc["hy"]) == (f32["hx"], f32["hy"]) == (2 * xs[0], 2 * ys[0])
    assert abs(ftc["ncc"] - f32["ncc"]) < 1e-6
    s.close()


@pytest.mark.parametrize("tw,th,w,h", [(64, 64, 3840, 2160), (32, 32, 16384, 256), (96, 96, 256, 16384)])
def test_tc_map_on_large_pictures(vtg_lib, ctx, tw, th, w, h):
    """A 4K picture and the widest and tallest pictures a search takes (16384 a side): the BF16 map within its bound of
    the F32 map, the same cells, and the template found where it was cut, with the F32 re-score's value."""
    frame = S.noise_frame(w, h, seed=w + 7 * h)
    tpl, xs, ys, blank = S.ncc_templates(frame, max(tw, th), 2, seed=5, blank_share=0.0)
    patch = tpl[0][:th, :tw].astype(np.float32)
    app = (patch - np.float32(patch.mean(dtype=np.float64))).astype(np.float32)
    norm = float(np.sum(app.astype(np.float64) ** 2))
    dp = _dev(frame)
    s = vtg_lib.Search(ctx, w, h, max_tw=128, max_th=128)
    s.template(app, norm)
    f32, v32, _, _ = s.run(dp.data_ptr(), w, h, w, vtg_lib.PLANE_U8, 1, w, 1, h, 1, vtg_lib.NCC_F32, want_map=True)
    ftc, vtc, _, _ = s.run(dp.data_ptr(), w, h, w, vtg_lib.PLANE_U8, 1, w, 1, h, 1, vtg_lib.NCC_BF16, want_map=True)
    assert ftc["cells"] == f32["cells"] and np.abs(vtc - v32).max() < TOL_MAP[1]
    assert (ftc["hx"], ftc["hy"]) == (f32["hx"], f32["hy"]) == (2 * xs[0], 2 * ys[0])
    assert abs(ftc["ncc"] - f32["ncc"]) < 1e-6
    s.close()


@pytest.mark.parametrize("precision", [1, 2])
def test_tc_step2_and_window(vtg_lib, ctx, precision):
    """A window that starts off the cell grid, at step 2, as the whole-picture band search runs at levels 0 and 1."""
    w, h = 500, 260
    frame = S.noise_frame(w, h, seed=77)
    tpl, xs, ys, _ = S.ncc_templates(frame, 32, 1, seed=9, blank_share=0.0)
    app = (tpl[0].astype(np.float32) - np.float32(tpl[0].mean(dtype=np.float64))).astype(np.float32)
    norm = float(np.sum(app.astype(np.float64) ** 2))
    dp = _dev(frame)
    s = vtg_lib.Search(ctx, w, h)
    s.template(app, norm)
    for (x0, x1, y0, y1, step) in ((37, 433, 5, 201, 2), (3, 499, 1, 259, 1), (40, 41, 40, 41, 1)):
        a, av, ax, ay = s.run(dp.data_ptr(), w, h, w, vtg_lib.PLANE_U8, x0, x1, y0, y1, step, vtg_lib.NCC_F32, True)
        b, bv, bx, by = s.run(dp.data_ptr(), w, h, w, vtg_lib.PLANE_U8, x0, x1, y0, y1, step, precision, True)
        assert a["cells"] == b["cells"] and np.abs(av - bv).max() < TOL_MAP[precision]
        clear = np.abs(av - bv) < 1e-7
        assert np.array_equal(ax[clear], bx[clear]) and np.array_equal(ay[clear], by[clear])
        assert (a["hx"], a["hy"]) == (b["hx"], b["hy"])
    s.close()


@pytest.mark.parametrize("step", [2, 4, 8, 16])
def test_steps_against_fp64_oracle(vtg_lib, ctx, step):
    """search_slot at every step the reference's band search uses: each candidate's half-pixel window of
    +-(2 step - 1), the second peak and the parabola, with the F32 and the tensor-core maps, against the FP64 oracle."""
    w, h, tw, th = 320, 240, 32, 24
    frame = S.noise_frame(w, h, seed=40 + step)
    tpl, xs, ys, _ = S.ncc_templates(frame, 32, 1, seed=step, blank_share=0.0)
    patch = tpl[0][:th, :tw].astype(np.float32)
    app = (patch - np.float32(patch.mean(dtype=np.float64))).astype(np.float32)
    norm = float(np.sum(app.astype(np.float64) ** 2))
    ref, _, _, _ = O.search_slot(frame.astype(np.float32), app, norm, 1, w, 1, h, step, mode=O.F64)
    dp = _dev(frame)
    s = vtg_lib.Search(ctx, w, h)
    s.template(app, norm)
    for prec in (vtg_lib.NCC_F32, vtg_lib.NCC_BF16, vtg_lib.NCC_FP16):
        f = s.run(dp.data_ptr(), w, h, w, vtg_lib.PLANE_U8, 1, w, 1, h, step, prec)
        assert (f["hx"], f["hy"]) == (ref["hx"], ref["hy"]), (prec, f, ref)
        assert abs(f["ncc"] - ref["ncc"]) < 1e-4 and abs(f["second"] - ref["second"]) < 1e-4
        assert abs(f["ox"] - ref["ox"]) < 2e-3 and abs(f["oy"] - ref["oy"]) < 2e-3
    s.close()


def test_window_without_corners(vtg_lib, ctx):
    """A window that the template cannot fit anywhere in: no candidates, nothing found, no kernel runs past the
    clamp."""
    w, h = 200, 100
    frame = S.noise_frame(w, h, seed=5)
    app = np.zeros((21, 32), np.float32)
    app[::2] = 1.0
    app -= app.mean()
    dp = _dev(frame)
    s = vtg_lib.Search(ctx, w, h)
    s.template(app, float(np.sum(app.astype(np.float64) ** 2)))
    for prec in (vtg_lib.NCC_F32, vtg_lib.NCC_BF16):
        f = s.run(dp.data_ptr(), w, h, w, vtg_lib.PLANE_U8, w - 20, w, 1, h, 1, prec)
        assert f["ntop"] == 0 and f["ncc"] == -2.0
    s.close()


def test_flat_picture_ties_across_ctas(vtg_lib, ctx):
    """A flat 1920 x 1080 picture: every window is near-blank, so every cell of every map scores exactly 0, and the
    eight candidates are the eight lowest cell indices (the reference's insertion order keeps the first of equal
    values), although each of the top-8 pass's CTAs offers a list of equal values. The F32 and the tensor-core paths
    then find the same corner with score 0."""
    w, h = 1920, 1080
    frame = np.full((h, w), 100, np.uint8)
    tpl, _, _, _ = S.ncc_templates(S.noise_frame(w, h, seed=6), 32, 1, seed=6, blank_share=0.0)
    app = (tpl[0].astype(np.float32) - np.float32(tpl[0].mean(dtype=np.float64))).astype(np.float32)
    norm = float(np.sum(app.astype(np.float64) ** 2))
    dp = _dev(frame)
    s = vtg_lib.Search(ctx, w, h)
    s.template(app, norm)
    found = []
    for prec in (vtg_lib.NCC_F32, vtg_lib.NCC_BF16, vtg_lib.NCC_FP16):
        f, v, mx, my = s.run(dp.data_ptr(), w, h, w, vtg_lib.PLANE_U8, 1, w, 1, h, 1, prec, True)
        assert f["cells"] > 4 * 1024  # the top-8 pass runs several CTAs
        assert np.all(v == 0.0) and not np.any(np.signbit(v)), prec
        assert f["ntop"] == 8 and f["ncc"] == 0.0, (prec, f)
        found.append((f["hx"], f["hy"], f["second"]))
    assert found[0] == found[1] == found[2]
    s.close()
