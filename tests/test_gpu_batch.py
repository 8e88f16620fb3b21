"""The batched form: many streams of uneven sizes in one step (one pyramid launch per level for all frames, one
persistent LK launch for all cells), graph capture and replay, and the autotuner.

Result invariance: every stream's cell records and lk_out records are the same bits in a batch as from that stream
alone (vtg_build + vtg_cells on its own tracker), whatever the batch's composition, launch shape or graph."""
import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu

SIZES = [(640, 480), (1280, 720), (1920, 1080), (640, 480), (960, 544), (1280, 720), (352, 288)]


def _pairs():
    out = []
    for k, (w, h) in enumerate(SIZES):
        f0, f1, _, _ = S.warp_pair(w, h, S.seeded_shift(40 + k, 0), 0.5, seed=40 + k)
        out.append((f0, f1))
    return out


def _single(vtg_lib, ctx, w, h, f0, f1, prev_cur=(0, 1)):
    t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=4))
    t.build(prev_cur[0], f0)
    t.build(prev_cur[1], f1)
    cells, lk = t.cells(*prev_cur)
    t.close()
    return cells, lk


@pytest.fixture(scope="module")
def batch_setup(vtg_lib, ctx):
    import torch

    pairs = _pairs()
    trackers = [vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=4)) for (w, h) in SIZES]
    dev = [(torch.from_numpy(f0).cuda(), torch.from_numpy(f1).cuda()) for f0, f1 in pairs]
    torch.cuda.synchronize()
    singles = [_single(vtg_lib, ctx, w, h, f0, f1) for (w, h), (f0, f1) in zip(SIZES, pairs)]
    b = vtg_lib.Batch(ctx, 16)
    yield pairs, trackers, dev, singles, b
    b.close()
    for t in trackers:
        t.close()


def _check(vtg_lib, trackers, singles):
    for t, (c_ref, l_ref) in zip(trackers, singles):
        c, l = vtg_lib.tracker_results(t)
        assert c.tobytes() == c_ref.tobytes() and l.tobytes() == l_ref.tobytes()


def test_batch_equals_single_streams(vtg_lib, ctx, batch_setup):
    pairs, trackers, dev, singles, b = batch_setup
    for t, (d0, _) in zip(trackers, dev):
        t.build(0, d0.data_ptr(), where=vtg_lib.DEVICE)
    ctx.sync()
    b.prepare(0, trackers, [d1.data_ptr() for _, d1 in dev], [1] * len(trackers))
    assert b.cells(0) == sum(t.cols * t.rows for t in trackers)
    b.launch(0)
    ctx.sync()
    _check(vtg_lib, trackers, singles)
    # the batched pyramid is the reference's, bit for bit
    for k in (2, 6):
        ref = O.pyramid(pairs[k][1], 4)
        for L in range(4):
            assert np.array_equal(trackers[k].level(1, L), ref[L])


@pytest.mark.parametrize("tune", [dict(persistent=1, block_warps=8, chunk=1, ctas_per_sm=2, tsmem=0, tiled=0),
                                  dict(persistent=1, block_warps=4, chunk=4, ctas_per_sm=4, tsmem=0, tiled=0),
                                  dict(persistent=0, block_warps=16, chunk=2, ctas_per_sm=1, tsmem=0, tiled=0),
                                  dict(persistent=1, block_warps=16, chunk=8, ctas_per_sm=1, tsmem=0, tiled=0),
                                  dict(persistent=1, block_warps=4, chunk=2, ctas_per_sm=5, tsmem=1, tiled=0),
                                  dict(persistent=1, block_warps=8, chunk=1, ctas_per_sm=3, tsmem=1, tiled=0),
                                  dict(persistent=1, block_warps=16, chunk=2, ctas_per_sm=1, tsmem=1, tiled=0),
                                  dict(persistent=1, block_warps=16, chunk=2, ctas_per_sm=1, tsmem=1, tiled=1),
                                  dict(persistent=1, block_warps=8, chunk=4, ctas_per_sm=2, tsmem=0, tiled=1),
                                  dict(persistent=1, block_warps=4, chunk=1, ctas_per_sm=5, tsmem=1, tiled=1)])
def test_batch_launch_shapes_do_not_change_results(vtg_lib, ctx, batch_setup, tune):
    """Every launch shape, the template in registers or in shared memory, cells in row order or in 8 x 4 tiles dealt
    to the CTAs, gives the single-stream bits."""
    pairs, trackers, dev, singles, b = batch_setup
    for t, (d0, _) in zip(trackers, dev):
        t.build(0, d0.data_ptr(), where=vtg_lib.DEVICE)
    b.set_tune(**tune)
    b.prepare(0, trackers, [d1.data_ptr() for _, d1 in dev], [1] * len(trackers))
    b.launch(0)
    ctx.sync()
    _check(vtg_lib, trackers, singles)


def test_batch_refuses_bad_tunes(vtg_lib, ctx, batch_setup):
    b = batch_setup[4]
    before = b.get_tune()
    for bad in (dict(persistent=1, block_warps=16, chunk=1, ctas_per_sm=2, tsmem=1, tiled=0),
                dict(persistent=0, block_warps=4, chunk=1, ctas_per_sm=1, tsmem=1, tiled=0),
                dict(persistent=1, block_warps=8, chunk=1, ctas_per_sm=4, tsmem=1, tiled=0),
                dict(persistent=1, block_warps=6, chunk=1, ctas_per_sm=1, tsmem=0, tiled=0),
                dict(persistent=1, block_warps=8, chunk=0, ctas_per_sm=1, tsmem=0, tiled=0),
                dict(persistent=0, block_warps=8, chunk=1, ctas_per_sm=1, tsmem=0, tiled=1),
                dict(persistent=1, block_warps=8, chunk=3, ctas_per_sm=1, tsmem=0, tiled=1)):
        with pytest.raises(vtg_lib.VtgError):
            b.set_tune(**bad)
    assert b.get_tune() == before


def test_batch_graph_replay_and_autotune(vtg_lib, ctx, batch_setup):
    pairs, trackers, dev, singles, b = batch_setup
    # slot 0: set 0 <- frame 0 ... slot 1: frame 1 into set 1, flow 0 -> 1; replay alternates them like a live stream
    b.prepare(0, trackers, [d0.data_ptr() for d0, _ in dev], [0] * len(trackers))
    b.prepare(1, trackers, [d1.data_ptr() for _, d1 in dev], [1] * len(trackers))
    b.capture(0)
    b.capture(1)
    for _ in range(3):
        b.replay(0)
        b.replay(1)
    ctx.sync()
    _check(vtg_lib, trackers, singles)
    best, best_ms, default_ms = b.autotune(1, reps=3)
    assert best_ms <= default_ms * 1.05 and best["block_warps"] in (4, 8, 16)
    b.launch(0)
    b.launch(1)
    ctx.sync()
    _check(vtg_lib, trackers, singles)


def test_batch_host_frames(vtg_lib, ctx, batch_setup):
    pairs, trackers, dev, singles, b = batch_setup
    b.prepare(0, trackers, [f0 for f0, _ in pairs], [0] * len(trackers), where=vtg_lib.HOST)
    b.prepare(1, trackers, [f1 for _, f1 in pairs], [1] * len(trackers), where=vtg_lib.HOST)
    b.launch(0)
    b.launch(1)
    ctx.sync()
    _check(vtg_lib, trackers, singles)


def test_batch_refuses_mixed_settings_and_repeats(vtg_lib, ctx, batch_setup):
    pairs, trackers, dev, singles, b = batch_setup
    other = vtg_lib.Tracker(ctx, vtg_lib.config(640, 480, levels=4, max_iter=5))
    with pytest.raises(vtg_lib.VtgError):
        b.prepare(0, [trackers[0], other], [dev[0][0].data_ptr(), dev[0][0].data_ptr()], [0, 0])
    with pytest.raises(vtg_lib.VtgError):
        b.prepare(0, [trackers[0], trackers[0]], [dev[0][0].data_ptr()] * 2, [0, 0])
    other.close()


def test_batch_at_its_maximum_of_512_streams(vtg_lib, ctx):
    """The largest batch (512 streams, the LK launch's job table at its limit) of small uneven frames, host frames,
    launched and replayed: every stream's cells equal its single-stream vtg_cells; a batch of 513 is refused."""
    import ctypes as C

    h = C.c_void_p()
    assert vtg_lib.lib().vtg_batch_create(ctx.h, 513, C.byref(h)) == vtg_lib.EINVAL
    sizes = [(32 + 8 * (k % 5), 32 + 4 * (k % 7)) for k in range(512)]
    frames = []
    for k, (w, h_) in enumerate(sizes):
        f0, f1, _, _ = S.warp_pair(w, h_, (0.7 + 0.01 * (k % 9), -0.4), 0.3, seed=1000 + k)
        frames.append((f0, f1))
    cfg = dict(levels=2, patch_w=7, patch_h=7, cell_w=8, cell_h=8)
    singles = []
    for (w, h_), (f0, f1) in zip(sizes[:64], frames[:64]):  # the single-stream results of a sample
        t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h_, **cfg))
        t.build(0, f0)
        t.build(1, f1)
        singles.append(t.cells(0, 1))
        t.close()
    trackers = [vtg_lib.Tracker(ctx, vtg_lib.config(w, h_, **cfg)) for (w, h_) in sizes]
    b = vtg_lib.Batch(ctx, 512)
    b.prepare(0, trackers, [f0 for f0, _ in frames], [0] * 512, where=vtg_lib.HOST)
    b.prepare(1, trackers, [f1 for _, f1 in frames], [1] * 512, where=vtg_lib.HOST)
    assert b.cells(1) == sum(t.cols * t.rows for t in trackers)
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
        _check(vtg_lib, trackers[:64], singles)
    # the rest against the oracle's pyramid and the single-stream code path once more, spread over the batch
    for k in range(64, 512, 37):
        t = vtg_lib.Tracker(ctx, vtg_lib.config(*sizes[k], **cfg))
        t.build(0, frames[k][0])
        t.build(1, frames[k][1])
        c_ref, l_ref = t.cells(0, 1)
        t.close()
        c, l = vtg_lib.tracker_results(trackers[k])
        assert c.tobytes() == c_ref.tobytes() and l.tobytes() == l_ref.tobytes(), k
        assert np.array_equal(trackers[k].level(1, 1), O.pyramid(frames[k][1], 2)[1])
    b.close()
    for t in trackers:
        t.close()


def test_batch_count(vtg_lib, ctx, batch_setup):
    """vtg_batch_count runs the step's LK launch once more with counters on: the work it reports bounds what the
    records say (forward iterations are lk_out.iters; every good track runs its backward walk), and the cells are
    the same bits after it."""
    pairs, trackers, dev, singles, b = batch_setup
    for t, (d0, _) in zip(trackers, dev):
        t.build(0, d0.data_ptr(), where=vtg_lib.DEVICE)
    ctx.sync()
    b.prepare(0, trackers, [d1.data_ptr() for _, d1 in dev], [1] * len(trackers))
    b.launch(0)
    ctx.sync()
    w = b.count(0)
    _check(vtg_lib, trackers, singles)
    lks = [vtg_lib.tracker_results(t)[1] for t in trackers]
    cells = sum(len(l) for l in lks)
    fwd_iters = sum(int(l["iters"].astype(np.int64).sum()) for l in lks)
    good = sum(int(((l["status"] == 0) | (l["status"] == vtg_lib.LK_FLOWBACK)).sum()) for l in lks)
    assert w["iterations"] > fwd_iters  # the backward walks' iterations come on top
    assert w["iterations"] <= 2 * 10 * 4 * cells
    assert good <= w["residuals"] <= 2 * cells
    assert cells <= w["builds"] <= 2 * 4 * cells
    assert w["passes"] <= w["iterations"]
