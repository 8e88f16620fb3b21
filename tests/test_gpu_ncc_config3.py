"""The whole-picture appearance search at the benchmark's NCC configuration: a seeded 1920 x 1080 8-bit frame,
templates of 32 x 32, 64 x 64 and 96 x 96 cut at seeded corners and perturbed (gain 0.8-1.2, offset +-20, noise
sigma 3), one in ten replaced by a near-blank patch (standard deviation below 2), searched at step 1 with the F32 map
and with the tensor-core maps (BF16 and FP16 products, F32 accumulation).

What each search must give:
  - every perturbed template is found at the corner it was cut from, in every precision, and the tensor-core maps find
    the F32 map's corner with the F32 re-score's value;
  - the found score is within 1e-4 of the FP64 oracle's score at that half-pixel corner;
  - the tensor-core map's cells are within the products' rounding of the F32 map's cells;
  - a near-blank template never matches: its best score stays below 0.5, the bar the reference's own near-blank test
    holds the correlation to (src/host/vt_ncc_check.c:63).
The reference's near-blank rule itself acts on windows (search_at, src/kern/track.c:184-206: a window whose variance is
at most the template's energy / 16 scores 0). It is checked on a copy of the frame with flat patches pasted in: every
cell of the map whose corners' windows all lie inside a flat patch holds exactly 0 in every precision, which goes
through the tensor-core path's exact 32-bit window sums and integer threshold."""
import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu

W, H = 1920, 1080
TEMPLATES = 10  # per size; one in ten near-blank
TOL_MAP = {1: 0.02, 2: 0.005}  # BF16, FP16: max |map value - F32 map value| (as the map tests)
TOL_FP64 = 1e-4


def _dev(a):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    torch.cuda.synchronize()
    return t


def _app(tpl):
    patch = tpl.astype(np.float32)
    app = (patch - np.float32(patch.mean(dtype=np.float64))).astype(np.float32)
    return app, float(np.sum(app.astype(np.float64) ** 2))


def _flat_frame(frame, size, seed):
    """The frame with six flat patches (a grey level +- 1.5, rounded: standard deviation below 2) of 2 T x 2 T pasted
    at seeded places; returns it and the patches' corners."""
    out = frame.copy()
    side = 2 * size
    u = S.uniform(seed, 900 + size, 6 * 3).reshape(6, 3)
    boxes = []
    for k in range(6):
        px = int(2 + np.floor(u[k, 0] * (W - side - 4)))
        py = int(2 + np.floor(u[k, 1] * (H - side - 4)))
        level = 40.0 + 170.0 * u[k, 2]
        flat = level + 1.5 * (S.uniform(seed, 950 + 10 * size + k, side * side).reshape(side, side) * 2.0 - 1.0)
        out[py:py + side, px:px + side] = S.to_u8(flat)
        boxes.append((px, py, side))
    return out, boxes


def _cells_inside(boxes, size, ccols, crows):
    """Map cells (step 1, window from corner (1, 1)) all of whose corners' windows lie inside one flat patch."""
    cells = []
    for cy in range(crows):
        for cx in range(ccols):
            x0, y0 = 1 + 16 * cx, 1 + 16 * cy
            for px, py, side in boxes:
                if x0 >= px and y0 >= py and x0 + 15 + size <= px + side and y0 + 15 + size <= py + side:
                    cells.append(cy * ccols + cx)
                    break
    return np.array(cells, np.int64)


@pytest.mark.parametrize("size", [32, 64, 96])
def test_config3_search(vtg_lib, ctx, size):
    frame = S.noise_frame(W, H, seed=3)
    tpl, xs, ys, blank = S.ncc_templates(frame, size, TEMPLATES, seed=size, blank_share=0.1)
    assert int(blank.sum()) == 1
    dp = _dev(frame)
    fplane = frame.astype(np.float32)
    s = vtg_lib.Search(ctx, W, H, max_tw=128, max_th=128)
    for k in range(TEMPLATES):
        app, norm = _app(tpl[k])
        if blank[k]:
            assert float(np.std(tpl[k].astype(np.float64))) < 2.0
        s.template(app, norm)
        f32, v32, _, _ = s.run(dp.data_ptr(), W, H, W, vtg_lib.PLANE_U8, 1, W, 1, H, 1, vtg_lib.NCC_F32, want_map=True)
        for prec in (vtg_lib.NCC_F32, vtg_lib.NCC_BF16, vtg_lib.NCC_FP16):
            if prec == vtg_lib.NCC_F32:
                f, v = f32, v32
            else:
                f, v, _, _ = s.run(dp.data_ptr(), W, H, W, vtg_lib.PLANE_U8, 1, W, 1, H, 1, prec, want_map=True)
                assert f["cells"] == f32["cells"]
                assert np.abs(v - v32).max() < TOL_MAP[prec], (size, k, prec)
            assert f["ncc"] <= 1.0 + 1e-6
            if blank[k]:
                assert f["ncc"] < 0.5, ("a near-blank template matched", size, k, prec, f["ncc"])
                continue
            assert (f["hx"], f["hy"]) == (2 * int(xs[k]), 2 * int(ys[k])), (size, k, prec, f)
            assert (f["hx"], f["hy"]) == (f32["hx"], f32["hy"])
            assert abs(f["ncc"] - f32["ncc"]) < 1e-6
            ref = O.ncc_half(fplane, app, norm, f["hx"], f["hy"], O.F64)
            assert abs(f["ncc"] - ref) < TOL_FP64, (size, k, prec, f["ncc"], ref)
    s.close()


@pytest.mark.parametrize("size", [32, 64, 96])
def test_config3_near_blank_windows_score_zero(vtg_lib, ctx, size):
    frame = S.noise_frame(W, H, seed=3)
    flat, boxes = _flat_frame(frame, size, seed=5)
    tpl, xs, ys, blank = S.ncc_templates(frame, size, 3, seed=size + 1, blank_share=0.0)
    dp = _dev(flat)
    s = vtg_lib.Search(ctx, W, H, max_tw=128, max_th=128)
    checked = 0
    for k in range(3):
        app, norm = _app(tpl[k])
        s.template(app, norm)
        maps = {}
        for prec in (vtg_lib.NCC_F32, vtg_lib.NCC_BF16, vtg_lib.NCC_FP16):
            f, v, mx, my = s.run(dp.data_ptr(), W, H, W, vtg_lib.PLANE_U8, 1, W, 1, H, 1, prec, want_map=True)
            maps[prec] = v
        ccols = (W - size - 2 - 1) // 16 + 1
        crows = (H - size - 2 - 1) // 16 + 1
        assert len(maps[vtg_lib.NCC_F32]) == ccols * crows
        inside = _cells_inside(boxes, size, ccols, crows)
        assert len(inside) > 0
        for prec, v in maps.items():
            assert np.all(v[inside] == 0.0), (size, k, prec, v[inside][v[inside] != 0.0][:5])
            assert not np.any(np.signbit(v[inside])), (size, k, prec)  # +0, the reference's 0, never -0
        checked += len(inside)
        # the oracle agrees that those windows are near-blank: the FP64 map over one such cell is 0 everywhere
        c = int(inside[0])
        x0, y0 = 1 + 16 * (c % ccols), 1 + 16 * (c // ccols)
        om = O.ncc_map(flat.astype(np.float32), app, norm, x0, x0 + 15, y0, y0 + 15, O.F64)
        assert np.all(om == 0.0)
    assert checked > 0
    s.close()
