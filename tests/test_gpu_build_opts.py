"""tk_build's optional input steps on the GPU (vtg_tracker_set_build): the contrast stretch (img_minmax + img_norm with
tk_build's x87 gain and offset) and the 5 x 5 binomial (img_gauss5) before the reduce, through vtg_build and through
batch steps. Bar: every level bit for bit, against the reference's own tk_build (tests/golden/build_opts.npz) and the
oracle."""
import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu

SETTINGS = [0, 1, 2, 3]  # neither, contrast, pre-gauss, both


def _levels(t, set_, n):
    return [t.level(set_, L) for L in range(n)]


def test_build_opts_against_reference_fixture(vtg_lib, ctx, golden):
    g = np.load(golden + "/build_opts.npz")
    for i, (kind, (w, h, seed)) in enumerate(zip(g["kinds"], g["dims"])):
        w, h = int(w), int(h)
        f = O.m1_image(w, h) if kind == "m1" else S.build_frame(str(kind), w, h, int(seed))
        assert O.fnv(f) == int(g["case%d_frame_fnv" % i])
        t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=3))
        for opts in SETTINGS:
            t.set_build(opts)
            assert t.build_flags == opts
            t.build(opts & 1, f)
            got = [O.fnv(p) for p in _levels(t, opts & 1, 3)]
            assert got == [int(v) for v in g["case%d_fnv" % i][opts]], (str(kind), opts)
        t.close()


@pytest.mark.parametrize("w,h,levels,lo,hi", [(333, 199, 4, 90, 150), (32, 32, 1, 0, 255), (1921, 1081, 4, 40, 41),
                                              (97, 61, 3, 7, 7), (1280, 720, 5, 0, 60), (35, 300, 2, 200, 255)])
def test_build_opts_against_oracle(vtg_lib, ctx, w, h, levels, lo, hi):
    """Odd sizes, one level, a flat frame (no range: gain 1), a two-value range, the top of the grey scale."""
    base = S.noise_frame(w, h, seed=w + h)
    f = (lo + (base.astype(np.int32) * (hi - lo + 1)) // 256).astype(np.uint8)
    t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=levels, cell_w=8, cell_h=8))
    for opts in SETTINGS:
        t.set_build(opts)
        t.build(1, f)
        want = O.pyramid(f, levels, opts)
        for L, (a, b) in enumerate(zip(_levels(t, 1, levels), want)):
            assert a.tobytes() == b.tobytes(), (opts, L)  # bits: the stretch can leave -0 at the minimum
    t.close()


def test_build_opts_frames_in_turn_strided_and_device(vtg_lib, ctx):
    """Frames of different ranges one after another into both sets (the min / max ticket is reused), a frame with a
    row pitch wider than its width, and a frame already in device memory."""
    import torch

    w, h = 640, 480
    t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=3))
    t.set_build(vtg_lib.BUILD_CONTRAST | vtg_lib.BUILD_PRE_GAUSS)
    for k, (lo, hi) in enumerate([(0, 255), (100, 140), (30, 31), (0, 0), (12, 250)]):
        f = (lo + (S.noise_frame(w, h, seed=70 + k).astype(np.int32) * (hi - lo + 1)) // 256).astype(np.uint8)
        wide = np.zeros((h, w + 48), np.uint8)
        wide[:, :w] = f
        t.build(k & 1, wide, stride=w + 48)
        want = O.pyramid(f, 3, 3)
        assert all(a.tobytes() == b.tobytes() for a, b in zip(_levels(t, k & 1, 3), want)), k
    f = S.build_frame("low", w, h, 9)
    d = torch.from_numpy(f).cuda()
    torch.cuda.synchronize()
    t.set_build(vtg_lib.BUILD_CONTRAST)
    t.build(0, d.data_ptr(), where=vtg_lib.DEVICE)
    assert all(a.tobytes() == b.tobytes() for a, b in zip(_levels(t, 0, 3), O.pyramid(f, 3, 1)))
    with pytest.raises(vtg_lib.VtgError):
        t.set_build(4)
    t.close()


def test_build_opts_in_batch_steps(vtg_lib, ctx):
    """A batch of trackers with every setting (and none) builds the same pyramids and cells as each tracker alone,
    launched and replayed from a captured graph."""
    import torch

    sizes = [(640, 480), (352, 288), (640, 480), (1280, 720)]
    opts = [1, 0, 3, 2]
    # frame 1 is frame 0 warped; both squeezed into grey 100 .. 140
    pairs = []
    for k, (w, h) in enumerate(sizes):
        f0, f1, _, _ = S.warp_pair(w, h, (1.3, -0.6), 0.3, seed=20 + k)
        pairs.append(tuple((100 + (f.astype(np.int32) * 40) // 255).astype(np.uint8) for f in (f0, f1)))
    singles = []
    for (w, h), o, (f0, f1) in zip(sizes, opts, pairs):
        t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=3))
        t.set_build(o)
        t.build(0, f0)
        t.build(1, f1)
        singles.append((_levels(t, 1, 3), t.cells(0, 1)))
        t.close()
    trackers = [vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=3)) for (w, h) in sizes]
    for t, o in zip(trackers, opts):
        t.set_build(o)
    dev = [(torch.from_numpy(f0).cuda(), torch.from_numpy(f1).cuda()) for f0, f1 in pairs]
    torch.cuda.synchronize()
    b = vtg_lib.Batch(ctx, 8)
    b.prepare(0, trackers, [d0.data_ptr() for d0, _ in dev], [0] * 4)
    b.prepare(1, trackers, [d1.data_ptr() for _, d1 in dev], [1] * 4)
    for replay in (False, True):
        if replay:
            b.capture(0)
            b.capture(1)
            b.replay(0)
            b.replay(1)
        else:
            b.launch(0)
            b.launch(1)
        ctx.sync()
        for k, t in enumerate(trackers):
            levels, (cells, lk) = singles[k]
            assert all(a.tobytes() == c.tobytes() for a, c in zip(_levels(t, 1, 3), levels)), (k, replay)
            assert all(a.tobytes() == c.tobytes() for a, c in zip(_levels(t, 1, 3), O.pyramid(pairs[k][1], 3, opts[k])))
            gc, gl = vtg_lib.tracker_results(t)
            assert gc.tobytes() == cells.tobytes() and gl.tobytes() == lk.tobytes(), (k, replay)
    b.close()
    for t in trackers:
        t.close()
