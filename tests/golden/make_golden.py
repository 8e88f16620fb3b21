"""make_golden.py -- writes the golden fixtures of tests/golden/ from the reference itself.

Run in a checkout that has the reference tree (it builds oracle/_ref from its sources):

    python tests/golden/make_golden.py [/root/reference]

Writes:
  m1_m2.json        the reference's committed gate logs: per-kernel plane hashes (logs/m1/host/m1-host-*.txt) and the
                    LK lines (logs/m2/host/640x480.txt), parsed.
  lk_640x480.npz    the 640 x 480 frame pair of the first benchmark configuration (seeded generator) and the reference's
                    lk_track_vx + lk_flowback_vx (and lk_track_ref + lk_flowback_ref) at its 1,200 cell centres.
  lk_1080p.npz      the 1920 x 1080 pair: the reference pyramid's per-level FNV hashes for both frames, and
                    lk_track_vx + lk_flowback_vx at every 8th of the 16,200 cells of the 16 x 8 grid and at every 4th
                    of the 4,080 cells at half resolution.
  still_vectors.npz the reference's still_vectors (15 x 15, one level, 6 iterations, flowback 0.25) on a 640 x 480 pair.
  ncc_32x21.npz     tk_correlate at 2,000 corners and search_slot (step 1 and 2) for a 32 x 21 template on a Q6 plane.
  detect.npz        corner detection (detect_begin, the three stages, detect_finish) over seven regions of two Q6
                    planes: each region's layout, a hash of its response map, its cells' strongest responses and the
                    corners found.
  still.npz         the still picture (still_vectors, still_decide, still_update, still_finish) over a 12-frame
                    320 x 240 sequence: per frame the cells after the decision, still_motion and still_hash.
  appearance.npz    store_appearance on two frames' pyramids, 60 regions each: validity, level, fraction, norm, hash.
  build_opts.npz    tk_build with the contrast stretch and / or the 5 x 5 binomial on six frames: per-level hashes.
  framegen.npz      frame generation (framegen.c as tk_generate_make runs it) on three pairs: the fields of every
                    level, the middle-instant field, hashes of the generated frame and its bytes, the scene verdict.
Frames are not stored: the generator reproduces them bit for bit, and their hashes are stored to prove it.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "intel-phi-visiontrack_gb300"))

import oracle as O  # noqa: E402
import vtg_synth as S  # noqa: E402


def parse_logs(ref_root: str) -> dict:
    m1 = {}
    for size in ("640x480", "1280x720", "1920x1080"):
        with open(os.path.join(ref_root, "logs", "m1", "host", "m1-host-%s.txt" % size)) as f:
            for line in f:
                m = re.match(r"kern (\S+)\s+(\d+)x(\d+) ([0-9a-f]{16})$", line.strip())
                if m:
                    m1["%s %s" % (m.group(1), size)] = m.group(4)
                m = re.match(r"kern minmax\s+(\d+)x(\d+) (\S+) (\S+)$", line.strip())
                if m:
                    m1["minmax " + size] = [float(m.group(3)), float(m.group(4))]
    m2 = []
    with open(os.path.join(ref_root, "logs", "m2", "host", "640x480.txt")) as f:
        for line in f:
            m2.append(line.rstrip("\n"))
    # the M2 pattern's accuracy against exact truth (docs/measurements.md, the table under "Displacement, px"):
    # displacement, points with status OK of 330, EPE median / p95 / max
    acc = []
    with open(os.path.join(ref_root, "docs", "measurements.md")) as f:
        lines = f.read().splitlines()
    start = next(i for i, line in enumerate(lines) if line.startswith("| Displacement, px"))
    for line in lines[start + 2:]:
        if not line.startswith("|"):
            break
        cols = [c.strip().strip("*") for c in line.strip("|").split("|")]
        d = [float(v) for v in cols[0].strip("()").split(",")]
        ok = int(cols[1].split("/")[0])
        acc.append({"d": d, "ok": ok, "median": float(cols[2]), "p95": float(cols[3]), "max": float(cols[4])})
    return {"m1": m1, "m2": m2, "m2_accuracy": acc}


def frames_1080():
    return S.warp_pair(1920, 1080, S.seeded_shift(2, 0), 0.5, seed=2)


def main(ref_root: str = "/root/reference") -> None:
    assert O.ref_available(), "oracle/_ref could not be built: the reference tree is needed"
    with open(os.path.join(HERE, "m1_m2.json"), "w") as f:
        json.dump(parse_logs(ref_root), f, indent=1)

    cfg = O.lk_cfg(21, 21, 10, 0.01, 0.1, 25.0)
    # configuration 1: 640 x 480, 3 levels, 16 x 16 grid
    f0, f1, _, _ = S.warp_pair(640, 480, (1.7, -0.8), 0.5, seed=1)
    xs, ys = O.cell_centres(640, 480, 16, 16)
    vx = O.ref_lk_points(f0, f1, 3, 2, cfg, xs, ys, max_fb=0.5)
    rf = O.ref_lk_points(f0, f1, 3, 2, cfg, xs, ys, max_fb=0.5, use_ref=True)
    np.savez_compressed(os.path.join(HERE, "lk_640x480.npz"), f0_fnv=np.uint64(O.fnv(f0)), f1_fnv=np.uint64(O.fnv(f1)),
                        xs=xs, ys=ys, vx=vx.view(np.uint8), ref=rf.view(np.uint8))

    # configuration 2: 1920 x 1080, 4 levels
    f0, f1, _, _ = frames_1080()
    p0 = O.ref_pyramid(f0, 4)
    p1 = O.ref_pyramid(f1, 4)
    xs, ys = O.cell_centres(1920, 1080, 16, 8)
    sel = np.arange(0, len(xs), 8)
    vx = O.ref_lk_points(f0, f1, 4, 3, cfg, xs[sel], ys[sel], max_fb=0.5)
    # half resolution: cells of 16 x 8 on level 1 (960 x 540), LK on levels 1..3
    hx, hy = O.cell_centres(960, 540, 16, 8)
    hsel = np.arange(0, len(hx), 4)
    hvx = O.ref_lk_points(f0, f1, 4, 2, cfg, hx[hsel], hy[hsel], max_fb=0.5, base=1)
    np.savez_compressed(os.path.join(HERE, "lk_1080p.npz"), f0_fnv=np.uint64(O.fnv(f0)), f1_fnv=np.uint64(O.fnv(f1)),
                        pyr0_fnv=np.array([O.fnv(p) for p in p0], np.uint64),
                        pyr1_fnv=np.array([O.fnv(p) for p in p1], np.uint64),
                        sel=sel.astype(np.int32), vx=vx.view(np.uint8), half_sel=hsel.astype(np.int32),
                        half_vx=hvx.view(np.uint8))

    # still_vectors, the reference's own per-cell flow (15 x 15, single level)
    g0, g1, _, _ = S.warp_pair(640, 480, (0.6, -0.3), 0.3, seed=5)
    sv = O.ref_still_vectors(g0, g1)
    np.savez_compressed(os.path.join(HERE, "still_vectors.npz"), f0_fnv=np.uint64(O.fnv(g0)),
                        f1_fnv=np.uint64(O.fnv(g1)), cells=sv.view(np.uint8))

    # the appearance correlation on a Q6 plane (level 0 of a synthetic frame)
    n0 = S.noise_frame(640, 480, seed=9)
    plane = O.pyramid(n0, 1)[0]
    app, norm = O.cut_template(plane, 300, 200, 32, 21)
    u = S.uniform(9, 77, 4000)
    cx = (1 + np.floor(u[:2000] * (640 - 32 - 3))).astype(np.int32)
    cy = (1 + np.floor(u[2000:] * (480 - 21 - 3))).astype(np.int32)
    cx[:9] = [300, 299, 301, 300, 300, 1, 606, 1, 606]
    cy[:9] = [200, 200, 200, 199, 201, 1, 1, 456, 456]
    corr = O.ref_correlate(plane, app, norm, cx, cy)
    f1s, mv1, mx1, my1 = O.ref_search_slot(plane, app, norm, 250, 360, 150, 260, 1)
    f2s, mv2, mx2, my2 = O.ref_search_slot(plane, app, norm, 1, 640, 1, 480, 2)
    hxs = np.array([2 * 300 + d for d in (-1, 0, 1, 0, 0, 1, -1)], np.int32)
    hys = np.array([2 * 200 + d for d in (0, 0, 0, -1, 1, 1, -1)], np.int32)
    half = O.ref_search_half(plane, app, norm, hxs, hys)
    np.savez_compressed(os.path.join(HERE, "ncc_32x21.npz"), frame_fnv=np.uint64(O.fnv(n0)), app=app,
                        norm=np.float32(norm), cx=cx, cy=cy, corr=corr,
                        s1=np.array([f1s["hx"], f1s["hy"]], np.int32), s1_ncc=f1s["ncc"], s1_second=f1s["second"],
                        s1_map_v=mv1, s1_map_x=mx1, s1_map_y=my1,
                        s2=np.array([f2s["hx"], f2s["hy"]], np.int32), s2_ncc=f2s["ncc"], s2_second=f2s["second"],
                        s2_map_v=mv2, s2_map_x=mx2, s2_map_y=my2, half_hx=hxs, half_hy=hys, half=half)
    # corner detection (detect.c) on Q6 planes: a textured 640 x 480 frame with a flat block, and a 1080p frame
    d0, _, _, _ = S.warp_pair(640, 480, (1.7, -0.8), 0.5, seed=1)
    d0 = d0.copy()
    d0[300:420, 40:200] = 128
    dplane = O.pyramid(d0, 1)[0]
    hplane = O.pyramid(f0, 1)[0]
    cases = [(0, 100.3, 80.7, 384, 307, 12, 128, 8.0, 0.05), (0, 0, 0, 640, 480, 12, 512, 6.0, 0.01),
             (0, 600, 400, 100, 100, 12, 64, 5.5, 0.1), (0, 17, 33, 50, 40, 4, 32, 3.0, 0.02),
             (0, 200.5, 150.25, 15, 10, 12, 16, 4.0, 0.05), (0, 50, 310, 140, 100, 12, 64, 5.0, 0.05),
             (1, 0, 0, 1920, 1080, 12, 512, 10.0, 0.01)]
    geo, resp_fnv, cells, cell_n, xs_all, ys_all, counts = [], [], [], [], [], [], []
    for (which, rx, ry, rw, rh, margin, mx, md, q) in cases:
        r = O.ref_detect(hplane if which else dplane, rx, ry, rw, rh, margin, mx, md, q)
        g, resp, cell, xs, ys = r
        geo.append([g[k] for k in ("x0", "y0", "x1", "y1", "ax", "cols", "rows", "nv", "cell_rows")])
        resp_fnv.append(O.fnv(resp))
        cells.append(cell.ravel())
        cell_n.append(cell.size)
        xs_all.append(xs)
        ys_all.append(ys)
        counts.append(len(xs))
    np.savez_compressed(os.path.join(HERE, "detect.npz"), frame_fnv=np.uint64(O.fnv(d0)),
                        frame1080_fnv=np.uint64(O.fnv(f0)), cases=np.array(cases, np.float64),
                        geo=np.array(geo, np.int32), resp_fnv=np.array(resp_fnv, np.uint64),
                        cells=np.concatenate(cells).astype(np.float32), cell_n=np.array(cell_n, np.int32),
                        xs=np.concatenate(xs_all).astype(np.float32), ys=np.concatenate(ys_all).astype(np.float32),
                        counts=np.array(counts, np.int32))
    write_still()
    write_framegen()
    write_build_opts()
    write_appearance()
    print("golden fixtures written to", HERE)


STILL_SEQ = dict(w=320, h=240, frames=12, seed=5, jump_at=9)
STILL_CFG = dict(avg=8, motion_px=1.0, motion_grey=4.0)


def write_still() -> None:
    """still.npz: the reference's still picture (still_vectors, still_decide, still_update, still_finish) over a
    12-frame 320 x 240 sequence: a drifting scene, sensor noise, a square moving in at frame 2, everything 40 grey
    brighter from frame 9. Per frame the cells after the decision, still_motion and still_hash."""
    frames = S.still_sequence(STILL_SEQ["w"], STILL_SEQ["h"], STILL_SEQ["frames"], STILL_SEQ["seed"],
                              jump_at=STILL_SEQ["jump_at"])
    cells, motion, hashes, mean = O.ref_still_run(frames, **STILL_CFG)
    np.savez_compressed(os.path.join(HERE, "still.npz"), frames_fnv=np.array([O.fnv(f) for f in frames], np.uint64),
                        seq=np.array([STILL_SEQ[k] for k in ("w", "h", "frames", "seed", "jump_at")], np.int64),
                        cfg=np.array([STILL_CFG["avg"], STILL_CFG["motion_px"], STILL_CFG["motion_grey"]], np.float64),
                        cells=cells, motion=motion, hashes=hashes, mean_fnv=np.uint64(O.fnv(mean)))


FG_CASES = [("pair", 640, 480, (6.3, 1.1), 3), ("odd", 333, 199, (-9.0, 5.5), 2), ("scene", 320, 240, (0.0, 0.0), 4)]


def write_framegen() -> None:
    """framegen.npz: the reference's frame generation (framegen.c, in tk_generate_make's order) on three pairs: every
    level's raw, filtered and upscaled fields, the middle-instant field, hashes of the frame and its bytes, the scene
    verdict."""
    out = {}
    for kind, w, h, shift, seed in FG_CASES:
        f0, f1 = S.framegen_pair("scene" if kind == "scene" else "pair", w, h, shift, seed)
        r = O.ref_framegen(f0, f1)
        out[kind + "_frames_fnv"] = np.array([O.fnv(f0), O.fnv(f1)], np.uint64)
        out[kind + "_scene"] = np.int32(r["scene"])
        for k in ("raw", "fil", "up"):
            out[kind + "_" + k] = np.concatenate([a.ravel() for a in r[k]])
        out[kind + "_mid"] = r["mid"].ravel()
        out[kind + "_out_fnv"] = np.uint64(O.fnv(r["out"]))
        out[kind + "_pic_fnv"] = np.uint64(O.fnv(r["pic"]))
    out["cases"] = np.array([(k == "scene", w, h, sx, sy, seed) for k, w, h, (sx, sy), seed in FG_CASES], np.float64)
    out["kinds"] = np.array([k for k, *_ in FG_CASES])
    np.savez_compressed(os.path.join(HERE, "framegen.npz"), **out)


BUILD_CASES = [("warp", 640, 480, 1), ("low", 640, 480, 2), ("flat", 160, 96, 0), ("dark", 208, 133, 4),
               ("low", 1920, 1080, 5)]


def write_build_opts() -> None:
    """build_opts.npz: the reference's tk_build with struct vt_config's contrast and pre_gauss (all four settings, x87
    and vector kernels alike) on the frames of vtg_synth.build_frame and the M1 gate's 640 x 480 frame: per case and
    setting, the FNV hash of every level (3 levels)."""
    out = {}
    frames = [("m1", 640, 480, 0, O.m1_image(640, 480))]
    frames += [(k, w, h, seed, S.build_frame(k, w, h, seed)) for k, w, h, seed in BUILD_CASES]
    for i, (kind, w, h, seed, f) in enumerate(frames):
        hashes = []
        for opts in range(4):
            planes = O.ref_tk_build(f, 3, opts, x87=True)
            vx = O.ref_tk_build(f, 3, opts, x87=False)
            assert all(a.tobytes() == b.tobytes() for a, b in zip(planes, vx)), (kind, opts)
            hashes.append([O.fnv(p) for p in planes])
        out["case%d_fnv" % i] = np.array(hashes, np.uint64)
        out["case%d_frame_fnv" % i] = np.uint64(O.fnv(f))
    out["kinds"] = np.array([k for k, *_ in frames])
    out["dims"] = np.array([(w, h, seed) for _, w, h, seed, _ in frames], np.int64)
    np.savez_compressed(os.path.join(HERE, "build_opts.npz"), **out)


APP_CASES = [(640, 480, 3, 1), (1920, 1080, 4, 2)]


def write_appearance() -> None:
    """appearance.npz: the reference's store_appearance on the pyramids its tk_build makes of two frames, for 60 seeded
    regions each (centres past the borders included): valid, level, fx, fy, norm and a hash of the template."""
    out = {}
    for i, (w, h, levels, seed) in enumerate(APP_CASES):
        f = S.build_frame("warp", w, h, seed)
        u = S.uniform(seed, 400, 4 * 60).reshape(60, 4)
        reg = np.stack([-20 + u[:, 0] * (w + 40), -20 + u[:, 1] * (h + 40), 10 + u[:, 2] * (w / 2 - 10),
                        10 + u[:, 3] * (h / 2 - 10)], 1).astype(np.float32)
        rows = []
        for cx, cy, rw, rh in reg:
            r = O.ref_store_appearance(f, levels, float(cx), float(cy), float(rw), float(rh))
            rows.append((r["valid"], r["level"] if r["valid"] else -1, r["fx"] if r["valid"] else 0.0,
                         r["fy"] if r["valid"] else 0.0, r["norm"] if r["valid"] else 0.0,
                         O.fnv(r["pix"]) if r["valid"] else 0))
        out["case%d_frame_fnv" % i] = np.uint64(O.fnv(f))
        out["case%d_regions" % i] = reg
        out["case%d_valid" % i] = np.array([r[0] for r in rows], np.int32)
        out["case%d_level" % i] = np.array([r[1] for r in rows], np.int32)
        out["case%d_f" % i] = np.array([(r[2], r[3], r[4]) for r in rows], np.float32)
        out["case%d_pix_fnv" % i] = np.array([r[5] for r in rows], np.uint64)
    out["cases"] = np.array(APP_CASES, np.int64)
    np.savez_compressed(os.path.join(HERE, "appearance.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
