"""Corner detection on the GPU (vtg_detect) against the reference's detect.c (tests/golden/detect.npz) and the oracle:
the region's layout, the response map and the cells bit for bit; the corners found, best first, equal to the
reference's."""
import os

import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    torch.cuda.synchronize()
    return t


def _planes():
    d0, _, _, _ = S.warp_pair(640, 480, (1.7, -0.8), 0.5, seed=1)
    d0 = d0.copy()
    d0[300:420, 40:200] = 128
    f0, _, _, _ = S.warp_pair(1920, 1080, S.seeded_shift(2, 0), 0.5, seed=2)
    return O.pyramid(d0, 1)[0], O.pyramid(f0, 1)[0]


def test_detect_against_reference_fixture(vtg_lib, ctx, golden):
    g = np.load(os.path.join(golden, "detect.npz"))
    planes = _planes()
    dev = [_dev(p) for p in planes]
    det = vtg_lib.Detector(ctx, 1920, 1080)
    c0 = p0 = 0
    for k, (which, rx, ry, rw, rh, margin, mx, md, q) in enumerate(g["cases"]):
        plane, dp = planes[int(which)], dev[int(which)]
        h, w = plane.shape
        xs, ys = det.detect(dp.data_ptr(), w, h, w, rx, ry, rw, rh, int(margin), int(mx), float(md), float(q))
        m = int(g["counts"][k])
        n = int(g["cell_n"][k])
        if m or n:
            geo, resp, cell = det.maps(rx, ry, rw, rh, w, h, int(margin))
            assert [geo[n_] for n_ in ("x0", "y0", "x1", "y1", "ax", "cols", "rows", "nv", "cell_rows")] == \
                list(g["geo"][k])
            assert O.fnv(resp) == int(g["resp_fnv"][k]), k
            assert np.array_equal(cell.ravel(), g["cells"][c0:c0 + n]), k
        c0 += n
        assert np.array_equal(xs, g["xs"][p0:p0 + m]) and np.array_equal(ys, g["ys"][p0:p0 + m]), k
        p0 += m
    det.close()


def test_detect_random_regions_against_oracle(vtg_lib, ctx):
    """Random rectangles, margins, spacings and qualities: maps bit for bit; corners as the oracle's (its scores in long
    double, the GPU's in FP64: equal unless two candidates' scores straddle an F32 rounding boundary)."""
    rng = np.random.default_rng(12)
    planes = [O.pyramid(S.noise_frame(320, 240, seed=s), 1)[0] for s in (3, 4)]
    planes.append(O.pyramid(O.m1_image(512, 384), 1)[0])
    dev = [_dev(p) for p in planes]
    det = vtg_lib.Detector(ctx, 512, 384)
    same = total = 0
    for _ in range(40):
        i = int(rng.integers(0, len(planes)))
        plane, dp = planes[i], dev[i]
        h, w = plane.shape
        rx, ry = float(rng.uniform(-20, w - 10)), float(rng.uniform(-20, h - 10))
        rw, rh = float(rng.uniform(5, w)), float(rng.uniform(5, h))
        margin, mx = int(rng.integers(3, 20)), int(rng.integers(1, 513))
        md, q = float(rng.uniform(1.0, 15.0)), float(rng.uniform(0.0, 0.2))
        xs, ys = det.detect(dp.data_ptr(), w, h, w, rx, ry, rw, rh, margin, mx, md, q)
        geo = O.detect_geometry(w, h, rx, ry, rw, rh, margin)
        if geo is None:
            assert len(xs) == 0
            continue
        rresp, rcell = O.detect_maps(plane, geo)
        _, resp, cell = det.maps(rx, ry, rw, rh, w, h, margin)
        assert np.array_equal(resp, rresp) and np.array_equal(cell, rcell)
        oxs, oys = O.detect(plane, rx, ry, rw, rh, margin, mx, md, q)
        total += 1
        if np.array_equal(xs, oxs) and np.array_equal(ys, oys):
            same += 1
        else:
            a = set(zip(xs.tolist(), ys.tolist()))
            b = set(zip(oxs.tolist(), oys.tolist()))
            assert len(a & b) >= 0.98 * max(len(a), len(b))
    assert same >= total - 1
    det.close()


def test_detect_on_a_tracker_level(vtg_lib, ctx):
    """The tracker's resident level 0 searched in place (the reseeding path of seed_at), against the oracle."""
    f0, _, _, _ = S.warp_pair(640, 480, (1.0, 0.5), 0.5, seed=8)
    t = vtg_lib.Tracker(ctx, vtg_lib.config(640, 480, levels=3))
    t.build(0, f0)
    t.sync()  # the detector's stream does not wait for the tracker's
    ptr, w, h, pitch = vtg_lib.level_device(t, 0, 0)
    det = vtg_lib.Detector(ctx, 640, 480)
    xs, ys = det.detect(ptr, w, h, pitch, 120.5, 90.25, 384, 307, 12, 128, 8.0, 0.05)
    oxs, oys = O.detect(O.pyramid(f0, 1)[0], 120.5, 90.25, 384, 307, 12, 128, 8.0, 0.05)
    assert len(xs) == 128 and np.array_equal(xs, oxs) and np.array_equal(ys, oys)
    det.close()
    t.close()


def test_detect_empty_and_refusals(vtg_lib, ctx):
    plane = O.pyramid(S.noise_frame(200, 100, seed=2), 1)[0]
    dp = _dev(plane)
    det = vtg_lib.Detector(ctx, 200, 100)
    # a rectangle wholly inside the margin, no corners wanted, and a flat picture: nothing found
    assert len(det.detect(dp.data_ptr(), 200, 100, 200, 190, 90, 50, 50, 12, 64, 4.0, 0.05)[0]) == 0
    assert len(det.detect(dp.data_ptr(), 200, 100, 200, 0, 0, 200, 100, 12, 0, 4.0, 0.05)[0]) == 0
    flat = _dev(np.full((100, 200), 8000.0, np.float32))
    assert len(det.detect(flat.data_ptr(), 200, 100, 200, 0, 0, 200, 100, 12, 64, 4.0, 0.05)[0]) == 0
    # more corners than detect_finish keeps, and a region larger than the detector
    with pytest.raises(vtg_lib.VtgError):
        det.detect(dp.data_ptr(), 200, 100, 200, 0, 0, 200, 100, 12, 513, 4.0, 0.05)
    big = _dev(np.zeros((300, 400), np.float32))
    with pytest.raises(vtg_lib.VtgError):
        det.detect(big.data_ptr(), 400, 300, 400, 0, 0, 400, 300, 12, 64, 4.0, 0.05)
    # regions that are not numbers are refused; infinite or astronomically far ones, and a negative margin, hold nothing
    with pytest.raises(vtg_lib.VtgError):
        det.detect(dp.data_ptr(), 200, 100, 200, float("nan"), 0, 50, 50, 12, 64, 4.0, 0.05)
    for reg in ((float("inf"), 0, 50, 50), (0, 0, float("inf"), 50), (-float("inf"), 0, 50, 50), (3e9, 0, 50, 50),
                (-3e9, -3e9, 6e9, 6e9)):
        assert len(det.detect(dp.data_ptr(), 200, 100, 200, *reg, 12, 64, 4.0, 0.05)[0]) == 0, reg
    assert len(det.detect(dp.data_ptr(), 200, 100, 200, 0, 0, 200, 100, -1, 64, 4.0, 0.05)[0]) == 0
    det.close()
