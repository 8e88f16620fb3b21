"""The oracle, pinned: this project's CPU restatement against the reference's own golden logs, against fixtures the
reference produced (tests/golden/make_golden.py), and, where the reference tree is here, against the reference's code
itself (oracle/_ref). No GPU."""
import json
import os
import platform

import numpy as np
import pytest

import oracle as O
import vtg_synth as S

X86 = platform.machine() in ("x86_64", "AMD64")
x86_only = pytest.mark.skipif(not X86, reason="the lane model's long double is the x87 format only on x86-64")


def _golden(golden, name):
    return np.load(os.path.join(golden, name))


@pytest.mark.parametrize("size", ["640x480", "1280x720", "1920x1080"])
def test_pyramid_matches_m1_logs(golden, size):
    """u8 -> Q6 and one reduce reproduce the reference's M1 gate hashes (logs/m1/host/m1-host-*.txt)."""
    with open(os.path.join(golden, "m1_m2.json")) as f:
        m1 = json.load(f)["m1"]
    w, h = map(int, size.split("x"))
    p = O.pyramid(O.m1_image(w, h), 2)
    assert "%016x" % O.fnv(p[0]) == m1["u8_to_q6 " + size]
    assert "%016x" % O.fnv(p[1]) == m1["reduce " + size]


@pytest.mark.parametrize("size", ["640x480", "1280x720", "1920x1080"])
def test_image_kernels_match_m1_logs(golden, size):
    """The M1 gate's other kernels on its Q6 frame reproduce its hash lines: img_norm with gain / offset (0.75, 512),
    img_minmax, img_gauss5, img_sobel (x and y) and img_absdiff of the frame and its binomial."""
    with open(os.path.join(golden, "m1_m2.json")) as f:
        m1 = json.load(f)["m1"]
    w, h = map(int, size.split("x"))
    q = O.pyramid(O.m1_image(w, h), 1)[0]
    g = O.gauss5(q)
    ix, iy = O.sobel(q)
    got = {"norm": O.norm(q, 0.75, 512.0), "gauss5": g, "sobel_x": ix, "sobel_y": iy, "absdiff": O.absdiff(q, g)}
    for k, plane in got.items():
        assert "%016x" % O.fnv(plane) == m1[k + " " + size], k
    assert list(O.minmax(q)) == m1["minmax " + size]


@pytest.mark.skipif(not (X86 and np.finfo(np.longdouble).nmant == 63), reason="x87 long double on x86-64 only")
def test_contrast_gain_is_x87():
    """tk_build's stretch gain and offset (track.c:603-614), formed by the oracle in exact integer arithmetic, equal the
    x87 extended computation rounded to F32 (numpy's long double on x86-64 is that format): every byte min / max pair
    (x 64, the Q6 planes tk_build stretches) and 20,000 other whole-number ranges below 2^24."""
    lo = np.repeat(np.arange(256), 256) * 64
    hi = np.tile(np.arange(256), 256) * 64
    keep = hi >= lo
    lo, hi = lo[keep], hi[keep]
    rng = np.random.default_rng(3)
    rlo = rng.integers(0, 1 << 24, 20000)
    rhi = np.minimum(rlo + rng.integers(0, 1 << 12, 20000) * rng.integers(1, 4096, 20000), (1 << 24) - 1)
    lo, hi = np.concatenate([lo, rlo]), np.concatenate([hi, rhi])
    span = (hi - lo).astype(np.longdouble)
    gain = np.where(span > 0, np.longdouble(16320) / np.where(span > 0, span, 1), np.longdouble(1))
    want = np.stack([gain.astype(np.float32), (-lo.astype(np.longdouble) * gain).astype(np.float32)], 1)
    got = np.stack([O.contrast_gain(a, b) for a, b in zip(lo, hi)])
    assert got.view(np.uint32).tobytes() == want.view(np.uint32).tobytes()


def build_cases(g):
    """(kind, frame, per-setting level hashes) of tests/golden/build_opts.npz, the frames regenerated."""
    for i, (kind, (w, h, seed)) in enumerate(zip(g["kinds"], g["dims"])):
        f = O.m1_image(int(w), int(h)) if kind == "m1" else S.build_frame(str(kind), int(w), int(h), int(seed))
        assert O.fnv(f) == int(g["case%d_frame_fnv" % i])
        yield str(kind), f, g["case%d_fnv" % i]


def test_build_opts_fixture(golden):
    """tk_build's optional input steps (contrast stretch, 5 x 5 binomial, both, neither) reproduce the reference's
    pyramids on six frames (tests/golden/build_opts.npz), every level bit for bit."""
    for kind, f, want in build_cases(_golden(golden, "build_opts.npz")):
        for opts in range(4):
            assert [O.fnv(p) for p in O.pyramid(f, 3, opts)] == [int(v) for v in want[opts]], (kind, opts)


@pytest.mark.skipif(not O.ref_available(), reason="the reference tree is not on this machine")
@pytest.mark.parametrize("w,h,lo,hi,seed", [(96, 64, 0, 255, 1), (112, 77, 30, 31, 2), (48, 41, 200, 255, 3),
                                            (256, 150, 0, 3, 4), (64, 33, 128, 128, 5)])
def test_build_opts_against_reference_code(w, h, lo, hi, seed):
    """The oracle's build options against the reference's own tk_build (x87 and vector kernels) on uniform noise in
    [lo, hi]: full range, two levels, the top edge, a tiny range, one level."""
    f = (lo + np.floor(S.uniform(seed, 300, w * h) * (hi - lo + 1))).astype(np.uint8).reshape(h, w)
    for opts in range(4):
        want = O.ref_tk_build(f, 3, opts, x87=True)
        assert [p.tobytes() for p in want] == [p.tobytes() for p in O.ref_tk_build(f, 3, opts, x87=False)]
        assert [p.tobytes() for p in O.pyramid(f, 3, opts)] == [p.tobytes() for p in want], opts


def appearance_cases(g):
    """(levels, pyramid planes, regions, fixture rows) of tests/golden/appearance.npz, the frames regenerated."""
    for i, (w, h, levels, seed) in enumerate(g["cases"]):
        f = S.build_frame("warp", int(w), int(h), int(seed))
        assert O.fnv(f) == int(g["case%d_frame_fnv" % i])
        yield int(levels), f, O.pyramid(f, int(levels)), g["case%d_regions" % i], i


def test_appearance_fixture(golden):
    """store_appearance (track.c:935-974) restated: validity, level, fraction, norm and template equal the reference's
    on 120 regions of two frames (tests/golden/appearance.npz)."""
    g = _golden(golden, "appearance.npz")
    for levels, f, P, regions, i in appearance_cases(g):
        for k, (cx, cy, rw, rh) in enumerate(regions):
            a = O.store_appearance(P, float(cx), float(cy), float(rw), float(rh))
            assert int(a["valid"]) == int(g["case%d_valid" % i][k]), (i, k)
            if a["valid"]:
                assert a["level"] == int(g["case%d_level" % i][k])
                fx, fy, norm = g["case%d_f" % i][k]
                assert (a["fx"], a["fy"]) == (fx, fy) and a["norm"].tobytes() == norm.tobytes()
                assert O.fnv(a["pix"]) == int(g["case%d_pix_fnv" % i][k])


@pytest.mark.skipif(not O.ref_available(), reason="the reference tree is not on this machine")
def test_appearance_against_reference_code():
    """The restatement against the reference's own store_appearance on 300 random regions of a 208 x 133 frame's
    two-level pyramid and of a low-contrast 640 x 480 frame stretched by tk_build's contrast step."""
    for (w, h, levels, kind) in ((208, 133, 2, "warp"), (640, 480, 3, "low")):
        f = S.build_frame(kind, w, h, 7)
        P = O.pyramid(f, levels)
        u = S.uniform(7, 500, 4 * 300).reshape(300, 4)
        for cx, cy, rw, rh in np.stack([-20 + u[:, 0] * (w + 40), -20 + u[:, 1] * (h + 40), 10 + u[:, 2] * w / 2,
                                        10 + u[:, 3] * h / 2], 1).astype(np.float32):
            a = O.store_appearance(P, float(cx), float(cy), float(rw), float(rh))
            r = O.ref_store_appearance(f, levels, float(cx), float(cy), float(rw), float(rh))
            assert a["valid"] == r["valid"]
            if a["valid"]:
                assert (a["level"], a["fx"], a["fy"]) == (r["level"], r["fx"], r["fy"])
                assert a["pix"].tobytes() == r["pix"].tobytes() and a["norm"].tobytes() == r["norm"].tobytes()


@x86_only
def test_lk_lane_matches_m2_logs(golden):
    """The lane-model LK reproduces the reference's M2 gate lines (logs/m2/host/640x480.txt) bit for bit: 10 exact
    displacements, 330 points each, raw bits of point 0 and a hash of all 330 lk_out records."""
    with open(os.path.join(golden, "m1_m2.json")) as f:
        m2 = json.load(f)["m2"]
    w, h = 640, 480
    cfg = O.lk_cfg(21, 21, 10, 0.005, 0.1, 40.0)
    margin = 40 + 21
    pts = [(x, y) for y in range(margin, h - margin, 24) for x in range(margin, w - margin, 24)]
    xs = np.array([p[0] for p in pts], np.float32)
    ys = np.array([p[1] for p in pts], np.float32)
    p0 = O.pyramid(O.m2_render(w, h, 2048, 2048), 4)
    cases = [(0, 0), (1, 0), (0, 1), (2, 2), (-3, 1), (5, -6), (13, 7), (-22, 17), (49, -30), (-101, 66)]
    lines = []
    bits = lambda f: int(np.float32(f).view(np.uint32))
    for dx, dy in cases:
        p1 = O.pyramid(O.m2_render(w, h, 2048 - dx, 2048 - dy), 4)
        out = O.lk_points(p0, p1, 3, cfg, xs, ys, mode=O.LANE)
        o = out[0]
        lines.append("lk_first %d,%d x %08x y %08x eig %08x res %08x cxx %08x cxy %08x cyy %08x it %u st %u" % (
            dx, dy, bits(o["x"]), bits(o["y"]), bits(o["min_eig"]), bits(o["residual"]), bits(o["cov_xx"]),
            bits(o["cov_xy"]), bits(o["cov_yy"]), o["iters"], o["status"]))
        lines.append("lk_hash %d,%d %016x" % (dx, dy, O.fnv(out)))
    assert lines == m2


def m2_case_stats(out, xs, ys, dx, dy):
    """The M2 gate's accuracy line (src/card/m2_gate.c:145-164): points with status OK, and the EPE median, p95 and max
    against the exact displacement (dx, dy) / 4, as epe[ok / 2], epe[ok * 95 / 100] of the sorted F32 errors."""
    ok = out["status"] == 0
    ex = out["x"].astype(np.float64) - (xs.astype(np.float64) + 0.25 * dx)
    ey = out["y"].astype(np.float64) - (ys.astype(np.float64) + 0.25 * dy)
    e64 = np.sqrt(ex * ex + ey * ey)[ok]
    e = np.sort(e64.astype(np.float32))
    n = len(e)
    return n, float(e[n // 2]), float(e[n * 95 // 100]), float(e64.max())


def m2_points():
    w, h, margin = 640, 480, 40 + 21
    pts = [(x, y) for y in range(margin, h - margin, 24) for x in range(margin, w - margin, 24)]
    return np.array([p[0] for p in pts], np.float32), np.array([p[1] for p in pts], np.float32)


@x86_only
def test_lk_lane_matches_m2_accuracy_table(golden):
    """The lane model reproduces the reference's accuracy table against exact truth (docs/measurements.md:93-104: ten
    quarter-pixel displacements of the M2 pattern, 330 points): status-OK counts, EPE median, p95 and max to the
    printed 4 decimals."""
    with open(os.path.join(golden, "m1_m2.json")) as f:
        table = json.load(f)["m2_accuracy"]
    cfg = O.lk_cfg(21, 21, 10, 0.005, 0.1, 40.0)
    xs, ys = m2_points()
    p0 = O.pyramid(O.m2_render(640, 480, 2048, 2048), 4)
    for row in table:
        dx, dy = int(round(4 * row["d"][0])), int(round(4 * row["d"][1]))
        p1 = O.pyramid(O.m2_render(640, 480, 2048 - dx, 2048 - dy), 4)
        n, med, p95, mx = m2_case_stats(O.lk_points(p0, p1, 3, cfg, xs, ys, mode=O.LANE), xs, ys, dx, dy)
        assert n == row["ok"], row
        assert ["%.4f" % v for v in (med, p95, mx)] == ["%.4f" % row[k] for k in ("median", "p95", "max")], row


def test_oracle_team_size_invariance():
    """The reference's race check is hash invariance across thread counts; the oracle's threaded cells and points
    (an atomic work counter, as the reference's team) give the same bits on 1, 2, 3 and 8 threads, in both
    arithmetics."""
    f0, f1, _, _ = S.warp_pair(320, 240, (2.3, -1.1), 0.5, seed=21)
    P0, P1 = O.pyramid(f0, 3), O.pyramid(f1, 3)
    cfg = O.lk_cfg()
    xs, ys = O.cell_centres(320, 240, 16, 16)
    for mode in (O.LANE, O.F64):
        base_pts = O.lk_points(P0, P1, 2, cfg, xs, ys, max_fb=0.5, mode=mode, threads=1)
        base_cells = O.cells(P0, P1, 2, cfg, 16, 8, max_fb=0.5, mode=mode, threads=1)
        for threads in (2, 3, 8):
            assert O.lk_points(P0, P1, 2, cfg, xs, ys, max_fb=0.5, mode=mode, threads=threads).tobytes() == \
                base_pts.tobytes()
            got = O.cells(P0, P1, 2, cfg, 16, 8, max_fb=0.5, mode=mode, threads=threads)
            assert all(a.tobytes() == b.tobytes() for a, b in zip(got, base_cells))


def test_m2_f64_accuracy_against_exact_truth():
    """The FP64 oracle recovers the M2 pattern's exact quarter-pixel displacements to within 0.05 px (the reference's
    own accuracy table, docs/measurements.md:93-104, reads EPE medians of 0.007-0.012 px)."""
    w, h = 640, 480
    cfg = O.lk_cfg(21, 21, 10, 0.005, 0.1, 40.0)
    xs, ys = np.meshgrid(np.arange(61, w - 61, 24, dtype=np.float32), np.arange(61, h - 61, 24, dtype=np.float32))
    xs, ys = xs.ravel(), ys.ravel()
    p0 = O.pyramid(O.m2_render(w, h, 2048, 2048), 4)
    for dx, dy in [(5, -6), (13, 7), (-22, 17)]:
        p1 = O.pyramid(O.m2_render(w, h, 2048 - dx, 2048 - dy), 4)
        out = O.lk_points(p0, p1, 3, cfg, xs, ys, mode=O.F64)
        ok = out["status"] == 0
        epe = np.hypot(out["x"] - xs - dx / 4.0, out["y"] - ys - dy / 4.0)[ok]
        assert ok.mean() > 0.95 and np.median(epe) < 0.05


def test_config1_fixture(golden):
    """640 x 480, 1,200 cells, 3 levels, flowback: the oracle against the reference's lk_track_vx / lk_track_ref."""
    g = _golden(golden, "lk_640x480.npz")
    f0, f1, _, _ = S.warp_pair(640, 480, (1.7, -0.8), 0.5, seed=1)
    assert O.fnv(f0) == int(g["f0_fnv"]) and O.fnv(f1) == int(g["f1_fnv"]), "the generator no longer reproduces"
    P0, P1 = O.pyramid(f0, 3), O.pyramid(f1, 3)
    cfg = O.lk_cfg()
    vx = g["vx"].view(O.LK_OUT)
    lane = O.lk_points(P0, P1, 2, cfg, g["xs"], g["ys"], max_fb=0.5, mode=O.LANE, threads=4)
    if X86:
        assert lane.tobytes() == vx.tobytes()
    f64 = O.lk_points(P0, P1, 2, cfg, g["xs"], g["ys"], max_fb=0.5, mode=O.F64, threads=4)
    ok = (f64["status"] == 0) & (vx["status"] == 0)
    assert (f64["status"] == vx["status"]).mean() >= 0.99
    err = np.maximum(np.abs(f64["x"] - vx["x"]), np.abs(f64["y"] - vx["y"]))[ok]
    assert err.max() < 1e-3
    ref = g["ref"].view(O.LK_OUT)  # the scalar reference differs from the lane model by rounding only
    ok2 = (ref["status"] == 0) & ok
    assert np.abs(ref["x"] - vx["x"])[ok2].max() < 1e-3


def test_config2_fixture(golden):
    """1920 x 1080, 4 levels: the oracle's pyramid against the reference's per-level hashes (bit-exact), and its LK at
    every 8th cell of the 16,200-cell grid and every 4th of the 4,080 half-resolution cells."""
    g = _golden(golden, "lk_1080p.npz")
    f0, f1, _, _ = S.warp_pair(1920, 1080, S.seeded_shift(2, 0), 0.5, seed=2)
    assert O.fnv(f0) == int(g["f0_fnv"]) and O.fnv(f1) == int(g["f1_fnv"])
    P0, P1 = O.pyramid(f0, 4), O.pyramid(f1, 4)
    assert [O.fnv(p) for p in P0] == [int(v) for v in g["pyr0_fnv"]]
    assert [O.fnv(p) for p in P1] == [int(v) for v in g["pyr1_fnv"]]
    cfg = O.lk_cfg()
    xs, ys = O.cell_centres(1920, 1080, 16, 8)
    sel = g["sel"]
    vx = g["vx"].view(O.LK_OUT)
    lane = O.lk_points(P0, P1, 3, cfg, xs[sel], ys[sel], max_fb=0.5, mode=O.LANE, threads=8)
    if X86:
        assert lane.tobytes() == vx.tobytes()
    hx, hy = O.cell_centres(960, 540, 16, 8)
    hsel = g["half_sel"]
    hvx = g["half_vx"].view(O.LK_OUT)
    hl = O.lk_points(P0[1:], P1[1:], 2, cfg, hx[hsel], hy[hsel], max_fb=0.5, mode=O.LANE, threads=8)
    if X86:
        assert hl.tobytes() == hvx.tobytes()
    f64 = O.lk_points(P0[1:], P1[1:], 2, cfg, hx[hsel], hy[hsel], max_fb=0.5, mode=O.F64, threads=8)
    ok = (f64["status"] == 0) & (hvx["status"] == 0)
    assert np.maximum(np.abs(f64["x"] - hvx["x"]), np.abs(f64["y"] - hvx["y"]))[ok].max() < 1e-3


def test_still_vectors_fixture(golden):
    """The per-cell grid restated (centre, clamp, LK, flowback, cell record) against the reference's still_vectors."""
    g = _golden(golden, "still_vectors.npz")
    f0, f1, _, _ = S.warp_pair(640, 480, (0.6, -0.3), 0.3, seed=5)
    assert O.fnv(f0) == int(g["f0_fnv"]) and O.fnv(f1) == int(g["f1_fnv"])
    ref = g["cells"].view(O.CELL)
    cfg = O.lk_cfg(15, 15, 6, 0.01, 0.1, 16.0)
    _, cl = O.cells(O.pyramid(f0, 1), O.pyramid(f1, 1), 0, cfg, 16, 8, max_fb=0.25, mode=O.LANE, threads=4)
    if X86:
        assert cl.tobytes() == ref.tobytes()
    assert np.array_equal(cl["diff"], ref["diff"])
    assert np.array_equal(cl["state"], ref["state"])


def test_ncc_fixture(golden):
    """search_at, search_half, the per-cell map and search_slot on a 32 x 21 template: the lane restatement against the
    reference (bit for bit on x86), the exact-sum FP64 form within 1e-5."""
    g = _golden(golden, "ncc_32x21.npz")
    n0 = S.noise_frame(640, 480, seed=9)
    assert O.fnv(n0) == int(g["frame_fnv"])
    plane = O.pyramid(n0, 1)[0]
    app, norm = O.cut_template(plane, 300, 200, 32, 21)
    assert np.array_equal(app, g["app"]) and np.float32(norm) == g["norm"]
    lane = np.array([O.ncc_at(plane, app, norm, int(x), int(y), O.LANE) for x, y in zip(g["cx"], g["cy"])])
    f64 = np.array([O.ncc_at(plane, app, norm, int(x), int(y), O.F64) for x, y in zip(g["cx"], g["cy"])])
    if X86:
        assert np.array_equal(lane, g["corr"])
    assert np.abs(f64 - g["corr"]).max() < 1e-5
    assert g["corr"][0] > 0.999999
    half = np.array([O.ncc_half(plane, app, norm, int(a), int(b), O.LANE) for a, b in zip(g["half_hx"], g["half_hy"])])
    if X86:
        assert np.array_equal(half, g["half"])
    for key, args in (("s1", (250, 360, 150, 260, 1)), ("s2", (1, 640, 1, 480, 2))):
        f, mv, mx, my = O.search_slot(plane, app, norm, *args, mode=O.LANE)
        assert [f["hx"], f["hy"]] == list(g[key])
        n = len(g[key + "_map_v"])
        assert np.array_equal(mx[:n], g[key + "_map_x"]) and np.array_equal(my[:n], g[key + "_map_y"])
        if X86:
            assert f["ncc"] == float(g[key + "_ncc"]) and f["second"] == float(g[key + "_second"])
            assert np.array_equal(mv[:n], g[key + "_map_v"])


def test_near_blank_never_matches():
    """vt_ncc_check's property (src/host/vt_ncc_check.c:17-63), restated: windows with under a few grey levels of noise
    never read 0.5 or more, nothing reads over 1, and the template itself reads 1."""
    rng = np.random.default_rng(7)
    app = rng.integers(6000, 10000, size=(21, 32)).astype(np.float32)
    app -= np.float32(app.sum(dtype=np.float64) / app.size)
    norm = float((app.astype(np.float64) ** 2).sum())
    worst = -2.0
    for level in (16320, 12800, 640):
        for step in (0, 1, 2, 4, 8, 16, 32, 64):
            for _ in range(40):
                pl = (level - (rng.integers(0, step + 1, size=(42, 64)) if step else np.zeros((42, 64), int))).astype(np.float32)
                for mode in (O.LANE, O.F64):
                    v = O.ncc_at(np.ascontiguousarray(pl), app, norm, 4, 4, mode)
                    worst = max(worst, v)
                    assert v <= 1.0 + 1e-9
    assert worst < 0.5
    pl = np.full((42, 64), 8000.0, np.float32)
    pl[4:25, 4:36] += app
    assert O.ncc_at(pl, app, norm, 4, 4, O.LANE) > 0.999 and O.ncc_at(pl, app, norm, 4, 4, O.F64) > 0.999


@pytest.mark.skipif(not O.ref_available(), reason="the reference tree is not on this machine")
@pytest.mark.parametrize("w,h", [(33, 47), (64, 64), (97, 61), (640, 480), (1281, 719)])
def test_pyramid_against_reference_code(w, h):
    """Odd and small sizes: the oracle's pyramid equals the reference's img_u8_to_q6 + img_reduce, both variants."""
    frame = S.noise_frame(w, h, seed=w * 7 + h)
    levels = 4 if min(w, h) >= 64 else 3
    mine = O.pyramid(frame, levels)
    for use_ref in (False, True):
        ref = O.ref_pyramid(frame, levels, use_ref=use_ref)
        for a, b in zip(mine, ref):
            assert np.array_equal(a, b)


@pytest.mark.skipif(not (O.ref_available() and X86), reason="needs the reference tree and x86-64")
def test_lk_edge_cases_against_reference_code():
    """Points at and past the borders (LK_OUT), a flat picture (LK_LOWEIG), guesses, and a larger patch: the lane
    restatement equals lk_track_vx + lk_flowback_vx bit for bit."""
    w, h = 200, 150
    f0, f1, _, _ = S.warp_pair(w, h, (2.5, -1.5), 0.5, seed=11)
    f1[:, :40] = 128  # a flat band
    f0[:, :40] = 128
    xs = np.array([5, 11, 12, 13, 100, 187, 188, 189, 195, 30, 60, 150, 100.25, 99.75], np.float32)
    ys = np.array([75, 75, 75, 75, 5, 75, 75, 75, 75, 75, 140, 12, 70.5, 71.125], np.float32)
    gx = np.linspace(-3, 3, len(xs)).astype(np.float32)
    gy = np.linspace(2, -2, len(xs)).astype(np.float32)
    for (pw, ph, levels) in ((21, 21, 3), (15, 15, 1), (9, 13, 2), (29, 31, 2)):
        cfg = O.lk_cfg(pw, ph, 10, 0.01, 0.1, 25.0)
        P0, P1 = O.pyramid(f0, levels), O.pyramid(f1, levels)
        for fb in (0.0, 0.5):
            mine = O.lk_points(P0, P1, levels - 1, cfg, xs, ys, gx, gy, max_fb=fb, mode=O.LANE)
            ref = O.ref_lk_points(f0, f1, levels, levels - 1, cfg, xs, ys, gx, gy, max_fb=fb, threads=1)
            assert mine.tobytes() == ref.tobytes(), (pw, ph, levels, fb)


def _detect_planes():
    """The detection fixture's two Q6 planes: a textured 640 x 480 frame with a flat block, and 1080p level 0."""
    d0, _, _, _ = S.warp_pair(640, 480, (1.7, -0.8), 0.5, seed=1)
    d0 = d0.copy()
    d0[300:420, 40:200] = 128
    f0, _, _, _ = S.warp_pair(1920, 1080, S.seeded_shift(2, 0), 0.5, seed=2)
    return d0, f0


def test_detect_fixture(golden):
    """The oracle's corner detection against the reference's (tests/golden/detect.npz): the region's layout, the
    response map and the cells bit for bit everywhere (F32 in the reference's operation order); the corners found bit
    for bit on x86-64, where long double is the reference's x87 format."""
    g = np.load(os.path.join(golden, "detect.npz"))
    d0, f0 = _detect_planes()
    assert O.fnv(d0) == int(g["frame_fnv"]) and O.fnv(f0) == int(g["frame1080_fnv"])
    planes = [O.pyramid(d0, 1)[0], O.pyramid(f0, 1)[0]]
    c0 = p0 = 0
    for k, (which, rx, ry, rw, rh, margin, mx, md, q) in enumerate(g["cases"]):
        plane = planes[int(which)]
        geo = O.detect_geometry(plane.shape[1], plane.shape[0], rx, ry, rw, rh, int(margin))
        gd = geo.as_dict()
        assert [gd[n] for n in ("x0", "y0", "x1", "y1", "ax", "cols", "rows", "nv", "cell_rows")] == list(g["geo"][k])
        resp, cell = O.detect_maps(plane, geo)
        assert O.fnv(resp) == int(g["resp_fnv"][k])
        n = int(g["cell_n"][k])
        assert np.array_equal(cell.ravel(), g["cells"][c0:c0 + n])
        c0 += n
        xs, ys = O.detect(plane, rx, ry, rw, rh, int(margin), int(mx), float(md), float(q))
        m = int(g["counts"][k])
        if X86:
            assert np.array_equal(xs, g["xs"][p0:p0 + m]) and np.array_equal(ys, g["ys"][p0:p0 + m]), k
        else:
            assert abs(len(xs) - m) <= max(1, m // 50)
        p0 += m


@pytest.mark.skipif(not (O.ref_available() and X86), reason="needs the reference tree and x86-64")
def test_detect_against_reference_code():
    """Random regions, margins, spacings and qualities over three planes: the oracle equals detect_begin, the three
    stages and detect_finish of the reference bit for bit."""
    rng = np.random.default_rng(12)
    planes = [O.pyramid(S.noise_frame(320, 240, seed=s), 1)[0] for s in (3, 4)]
    planes.append(O.pyramid(O.m1_image(512, 384), 1)[0])
    for _ in range(40):
        plane = planes[int(rng.integers(0, len(planes)))]
        h, w = plane.shape
        rx, ry = float(rng.uniform(-20, w - 10)), float(rng.uniform(-20, h - 10))
        rw, rh = float(rng.uniform(5, w)), float(rng.uniform(5, h))
        margin, mx = int(rng.integers(3, 20)), int(rng.integers(1, 513))
        md, q = float(rng.uniform(1.0, 15.0)), float(rng.uniform(0.0, 0.2))
        ref = O.ref_detect(plane, rx, ry, rw, rh, margin, mx, md, q)
        geo = O.detect_geometry(w, h, rx, ry, rw, rh, margin)
        if ref is None:
            assert geo is None
            continue
        rg, rresp, rcell, rxs, rys = ref
        resp, cell = O.detect_maps(plane, geo)
        assert np.array_equal(resp, rresp) and np.array_equal(cell, rcell)
        xs, ys = O.detect(plane, rx, ry, rw, rh, margin, mx, md, q)
        assert np.array_equal(xs, rxs) and np.array_equal(ys, rys)


def _still_frames(g):
    w, h, n, seed, jump = (int(v) for v in g["seq"])
    frames = S.still_sequence(w, h, n, seed, jump_at=jump)
    assert [O.fnv(f) for f in frames] == [int(v) for v in g["frames_fnv"]]
    return frames


@x86_only
def test_still_fixture(golden):
    """The oracle's still picture (its per-cell grid in the lane model, then still_decide, still_update, still_finish)
    reproduces the reference's still_hash on every frame of the fixture: a drifting scene, a square moving in, the
    counts reaching avg, and a frame where everything changed."""
    g = _golden(golden, "still.npz")
    avg, px, grey = g["cfg"]
    frames = _still_frames(g)
    st = O.Still(frames[0].shape[1], frames[0].shape[0], int(avg), float(px), float(grey))
    for k, f in enumerate(frames):
        cells, m = st.frame(O.pyramid(f, 1)[0])
        assert O.still_hash(cells, st.mean) == int(g["hashes"][k]), k
        assert m.tobytes() == g["motion"][k].tobytes(), k
    assert O.fnv(st.mean) == int(g["mean_fnv"])
    assert int(g["motion"]["moving"][int(g["seq"][4])]) == len(cells)  # the frame where everything changed
    st.close()


def test_still_decision_on_reference_cells(golden):
    """still_decide and still_update alone, fed the reference's own vectors of each frame: the reference's hash on
    every frame, on any host (the decision's long double steps are exact or far from a rounding boundary here)."""
    g = _golden(golden, "still.npz")
    avg, px, grey = g["cfg"]
    frames = _still_frames(g)
    st = O.Still(frames[0].shape[1], frames[0].shape[0], int(avg), float(px), float(grey))
    for k, f in enumerate(frames):
        cells, m = st.frame(O.pyramid(f, 1)[0], cells=g["cells"][k])
        assert O.still_hash(cells, st.mean) == int(g["hashes"][k]), k
        assert np.array_equal(cells["state"], g["cells"][k]["state"])
    st.close()


@pytest.mark.skipif(not (O.ref_available() and X86), reason="needs the reference tree and x86-64")
@pytest.mark.parametrize("w,h,frames,avg,px,grey", [(200, 120, 7, 3, 0.5, 2.0), (129, 77, 5, 16, 2.0, 6.0)])
def test_still_against_reference_code(w, h, frames, avg, px, grey):
    """Other sizes (a ragged last cell row and column), averaging depths and gates, against still.c itself."""
    seq = S.still_sequence(w, h, frames, seed=11, jump_at=frames - 1, mover=16)
    _, rm, rh, rmean = O.ref_still_run(seq, avg, px, grey)
    st = O.Still(w, h, avg, px, grey)
    for k, f in enumerate(seq):
        cells, m = st.frame(O.pyramid(f, 1)[0])
        assert O.still_hash(cells, st.mean) == int(rh[k]), k
        assert m.tobytes() == rm[k].tobytes(), k
    assert np.array_equal(st.mean, rmean)
    st.close()


def fg_cases(g):
    """The fixture's pairs: (kind, frames)."""
    out = []
    for kind, (scene, w, h, sx, sy, seed) in zip(g["kinds"], g["cases"]):
        f0, f1 = S.framegen_pair("scene" if scene else "pair", int(w), int(h), (float(sx), float(sy)), int(seed))
        assert [O.fnv(f0), O.fnv(f1)] == [int(v) for v in g[str(kind) + "_frames_fnv"]]
        out.append((str(kind), f0, f1))
    return out


def test_framegen_fixture(golden):
    """The oracle's frame generation reproduces the reference's framegen.c (tests/golden/framegen.npz) on every pair:
    each level's raw, filtered and upscaled field, the middle-instant field, the frame, its bytes, the verdict."""
    g = _golden(golden, "framegen.npz")
    for kind, f0, f1 in fg_cases(g):
        r = O.framegen(O.pyramid(f0, 1)[0], O.pyramid(f1, 1)[0])
        assert r["scene"] == int(g[kind + "_scene"]), kind
        for k in ("raw", "fil", "up"):
            assert np.array_equal(np.concatenate([a.ravel() for a in r[k]]), g[kind + "_" + k]), (kind, k)
        assert np.array_equal(r["mid"].ravel(), g[kind + "_mid"]), kind
        assert O.fnv(r["out"]) == int(g[kind + "_out_fnv"]) and O.fnv(r["pic"]) == int(g[kind + "_pic_fnv"]), kind
    assert int(g["scene_scene"]) == 1 and int(g["pair_scene"]) == 0


@pytest.mark.skipif(not O.ref_available(), reason="the reference tree is not on this machine")
@pytest.mark.parametrize("w,h,shift,amp,seed", [(256, 192, (30.0, -22.0), 2.0, 5), (401, 257, (-1.2, 0.4), 0.0, 6),
                                                (130, 66, (4.5, 7.5), 1.0, 7), (800, 600, (-17.0, 12.0), 3.0, 8),
                                                (64, 64, (10.0, -7.0), 1.0, 9), (128, 96, (40.0, 30.0), 4.0, 10),
                                                (96, 200, (-45.0, 60.0), 0.0, 11)])
def test_framegen_against_reference_code(w, h, shift, amp, seed):
    """Shifts past the finest level's reach (found through the coarse levels), no motion, small and odd sizes."""
    f0, f1, _, _ = S.warp_pair(w, h, shift, amp, seed=seed)
    r = O.ref_framegen(f0, f1)
    o = O.framegen(O.pyramid(f0, 1)[0], O.pyramid(f1, 1)[0])
    assert r["scene"] == o["scene"]
    for k in ("raw", "fil", "up"):
        for a, b in zip(r[k], o[k]):
            assert np.array_equal(a, b), k
    for k in ("mid", "out", "pic"):
        assert np.array_equal(r[k], o[k]), k
