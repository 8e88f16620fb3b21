"""The served request loop (vtg_serve_run): Poisson arrivals from streams of mixed sizes, admission by device-memory
budget (streams wait for memory and are admitted as others finish), continuous batching with two batches in flight,
2 % of frame pairs followed by an appearance search; and the plain one-pair-at-a-time form for comparison."""
import pytest

import vtg_synth as S

pytestmark = pytest.mark.gpu


def _frames(sizes):
    import torch

    bufs = []
    for k, (w, h) in enumerate(sizes):
        f0, f1, _, _ = S.warp_pair(w, h, S.seeded_shift(70 + k, 0), 0.5, seed=70 + k)
        for f in (f0, f1):
            bufs.append(torch.from_numpy(f).pin_memory())
    return bufs


@pytest.mark.parametrize("plain", [False, True])
def test_serve_all_requests(vtg_lib, ctx, plain):
    sizes = [(640, 480), (1280, 720), (1920, 1080), (640, 480), (960, 544), (1920, 1080)]
    bufs = _frames(sizes)
    streams = [dict(width=w, height=h, flow_level=1 if w == 1920 else 0, fps=120.0, start_s=0.02 * k, frames=20)
               for k, (w, h) in enumerate(sizes)]
    lk = vtg_lib.config(64, 64, levels=4)
    st = vtg_lib.serve(ctx, streams, [b.data_ptr() for b in bufs], lk, duration_s=1.0, ncc_share=0.1, plain=plain)
    assert st["served"] == st["requests"] == 120
    assert st["streams_admitted"] == 6 and st["streams_rejected"] == 0
    assert 0.0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"] < 1000.0
    cells = sum(((w >> (1 if w == 1920 else 0)) + 15) // 16 * (((h >> (1 if w == 1920 else 0)) + 7) // 8) * 20
                for (w, h) in sizes)
    assert st["cells"] == cells
    if plain:
        assert st["mean_batch"] == 1.0


def test_serve_admission_waits_for_memory(vtg_lib, ctx):
    """A budget for two 1080p trackers at a time: the later streams wait, and are admitted as earlier ones finish."""
    sizes = [(1920, 1080)] * 4
    bufs = _frames(sizes)
    lk = vtg_lib.config(64, 64, levels=4)
    one = vtg_lib.lib().vtg_tracker_bytes(__import__("ctypes").byref(vtg_lib.config(1920, 1080, levels=4)))
    streams = [dict(width=1920, height=1080, fps=200.0, start_s=0.0, frames=10) for _ in sizes]
    st = vtg_lib.serve(ctx, streams, [b.data_ptr() for b in bufs], lk, duration_s=1.0, hbm_budget=2 * one + 1024)
    assert st["served"] == 40 and st["streams_admitted"] == 4 and st["streams_waited"] >= 2


@pytest.mark.parametrize("plain", [False, True])
def test_serve_results_same_alone_and_in_mix(vtg_lib, ctx, plain):
    """Each stream's results from the served loop are the bits its own tracker gives alone. The loop batches the
    streams together and pipelines each stream's consecutive frame pairs across the two slots (the later one waits
    on the GPU for the earlier one), so this holds the batching and that ordering to the single-stream result."""
    import numpy as np

    sizes = [(640, 480), (1280, 720), (1920, 1080), (960, 544)]
    flow = [1 if w == 1920 else 0 for w, _ in sizes]
    bufs = _frames(sizes)
    streams = [dict(width=w, height=h, flow_level=fl, fps=2000.0, start_s=0.0, frames=12)
               for (w, h), fl in zip(sizes, flow)]
    last = []
    for (w, h), fl in zip(sizes, flow):
        t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=4, flow_level=fl))
        last.append(np.zeros(t.cols * t.rows, vtg_lib.CELL_DTYPE))
        t.close()
    lk = vtg_lib.config(64, 64, levels=4)
    st = vtg_lib.serve(ctx, streams, [b.data_ptr() for b in bufs], lk, duration_s=1.0, plain=plain, last_cells=last)
    assert st["served"] == 48
    if not plain:
        assert st["mean_batch"] > 1.0
    for k, ((w, h), fl) in enumerate(zip(sizes, flow)):
        # the 12th pair: frame 1 in set 1 (from the 11th pair), frame 0 rebuilt into set 0, cells from set 1 to set 0
        t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=4, flow_level=fl))
        t.build(1, bufs[2 * k + 1].numpy())
        t.build(0, bufs[2 * k].numpy())
        cells, _ = t.cells(1, 0)
        t.close()
        assert np.array_equal(cells.view(np.uint8), last[k].view(np.uint8)), (w, h)
