"""The request API of the served loop (vtg_server_*): frames pushed as they arrive, cells polled back.

  - Result invariance with LIVE skips: four streams of mixed sizes, two of them LIVE, each handed a burst of frames at
    once. The ORDERED streams serve every frame; a LIVE stream serves its newest queued frame and reports the older ones
    as skipped, counted on the next served result (the card session's rule, src/card/session_track.c:199-205). Every
    served frame's cells are the bits a tracker alone gives for the pair (the last frame served for that stream, this
    frame), bit for bit.
  - Host-side faults, injected on the host (src/card/session_track.c:1031-1043 is the precedent): a malformed stream is
    refused and the server goes on; a stream that stops sending is retired after the idle bound and its memory goes back
    to the budget; a producer that stalls ends the Poisson driver with VTG_ETIMEOUT once every frame on the GPU has
    delivered its result; a malformed stream description in the driver is refused while the other streams run."""
import numpy as np
import pytest

import vtg_synth as S

pytestmark = pytest.mark.gpu


def _seq(w, h, n, seed):
    """n + 1 frames of a scene moving 0.7 px right and 0.4 px up a frame (uint8, pinned)."""
    import torch

    base = S.blurred_noise(w, h, seed)
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float64)
    out = []
    for k in range(n + 1):
        img = S.bilinear(base, xs - 0.7 * k, ys + 0.4 * k)
        out.append(torch.from_numpy(S.to_u8(img)).pin_memory())
    return out


def _alone(vtg_lib, ctx, w, h, fl, a, b):
    t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=4, flow_level=fl))
    t.build(0, a.numpy())
    t.build(1, b.numpy())
    cells, _ = t.cells(0, 1)
    t.close()
    return cells


def _drain(srv, want, limit_s=20.0):
    import time

    got, t0 = [], time.time()
    while len(got) < want and time.time() - t0 < limit_s:
        got += srv.poll(256, timeout_us=2000)
    return got


def test_server_live_skips_and_results_same_alone(vtg_lib, ctx):
    specs = [(640, 480, 0, vtg_lib.PRIO_LIVE), (1280, 720, 0, vtg_lib.PRIO_ORDERED),
             (1920, 1080, 1, vtg_lib.PRIO_LIVE), (960, 544, 0, vtg_lib.PRIO_ORDERED)]
    n = 5
    seqs = [_seq(w, h, n, seed=120 + k) for k, (w, h, _, _) in enumerate(specs)]
    srv = vtg_lib.Server(ctx, vtg_lib.config(64, 64, levels=4), max_batch=8, inflight=2, max_queue=16)
    ids, bufs, tickets = [], {}, {}
    for (w, h, fl, prio), seq in zip(specs, seqs):
        sid = srv.open(w, h, seq[0].data_ptr(), flow_level=fl, priority=prio)
        assert sid >= 0
        ids.append(sid)
    for k, ((w, h, fl, prio), seq) in enumerate(zip(specs, seqs)):
        t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=4, flow_level=fl))
        ncell = t.cols * t.rows
        t.close()
        for i in range(1, n + 1):
            cells = np.zeros(ncell, vtg_lib.CELL_DTYPE)
            tk = srv.submit(ids[k], seq[i].data_ptr(), cells, tag=100 * k + i)
            assert tk >= 0
            bufs[tk] = cells
            tickets[tk] = (k, i)
    res = _drain(srv, len(tickets))
    assert len(res) == len(tickets) and srv.pending() == 0
    steps, frames = srv.counts()
    assert frames > steps  # frames of several streams went together
    by_stream = {}
    for r in sorted(res, key=lambda r: r["ticket"]):
        by_stream.setdefault(tickets[r["ticket"]][0], []).append(r)
    for k, (w, h, fl, prio) in enumerate(specs):
        rs = by_stream[k]
        assert [tickets[r["ticket"]][1] for r in rs] == list(range(1, n + 1))
        skipped = [r for r in rs if r["status"] == vtg_lib.RES_SKIPPED]
        if prio == vtg_lib.PRIO_ORDERED:
            assert not skipped
        else:
            assert len(skipped) >= 1  # the burst was queued before the first step
        prev, run = 0, 0
        for r in rs:
            i = tickets[r["ticket"]][1]
            if r["status"] == vtg_lib.RES_SKIPPED:
                run += 1
                continue
            assert r["status"] == vtg_lib.RES_DONE and r["frames_skipped"] == run
            want = _alone(vtg_lib, ctx, w, h, fl, seqs[k][prev], seqs[k][i])
            assert np.array_equal(want.view(np.uint8), bufs[r["ticket"]].view(np.uint8)), (k, i)
            prev, run = i, 0
    srv.close()


def test_server_refuses_malformed_streams_and_goes_on(vtg_lib, ctx):
    import torch

    f = torch.from_numpy(S.noise_frame(640, 480, seed=4)).pin_memory()
    srv = vtg_lib.Server(ctx, vtg_lib.config(64, 64, levels=4))
    assert srv.open(16, 16, f.data_ptr()) == vtg_lib.EINVAL  # below the smallest picture
    assert srv.open(640, 480, f.data_ptr(), flow_level=7) == vtg_lib.EINVAL  # past the pyramid
    assert srv.open(640, 480, f.data_ptr(), priority=9) == vtg_lib.EINVAL
    sid = srv.open(640, 480, f.data_ptr())
    assert sid >= 0
    assert srv.submit(sid + 17, f.data_ptr()) == vtg_lib.EINVAL  # an unknown stream
    assert srv.submit(sid, f.data_ptr(), tag=5) >= 0
    res = _drain(srv, 1)
    assert len(res) == 1 and res[0]["status"] == vtg_lib.RES_DONE and res[0]["tag"] == 5
    srv.close()


def test_server_retires_a_stream_that_stops_sending(vtg_lib, ctx):
    import time

    import torch

    a = torch.from_numpy(S.noise_frame(640, 480, seed=5)).pin_memory()
    b = torch.from_numpy(S.noise_frame(1280, 720, seed=6)).pin_memory()
    srv = vtg_lib.Server(ctx, vtg_lib.config(64, 64, levels=4), idle_timeout_s=0.3)
    sa = srv.open(640, 480, a.data_ptr())
    sb = srv.open(1280, 720, b.data_ptr())
    assert sa >= 0 and sb >= 0
    bytes_a = vtg_lib.lib().vtg_tracker_bytes(__import__("ctypes").byref(vtg_lib.config(640, 480, levels=4)))
    used_both = ctx.used()
    srv.submit(sa, a.data_ptr())
    retired, done, t0 = [], 0, time.time()
    while time.time() - t0 < 5.0 and not retired:
        srv.submit(sb, b.data_ptr())  # stream b keeps sending, a has stopped
        for r in srv.poll(64, timeout_us=20000):
            if r["status"] == vtg_lib.RES_RETIRED:
                retired.append(r["stream"])
            else:
                done += 1
    assert retired == [sa] and done >= 2
    assert used_both - ctx.used() == bytes_a  # a's memory is back in the budget
    assert srv.submit(sa, a.data_ptr()) == vtg_lib.EINVAL  # a is closed
    srv.close()


def _frames(sizes, seed0):
    import torch

    bufs = []
    for k, (w, h) in enumerate(sizes):
        f0, f1, _, _ = S.warp_pair(w, h, S.seeded_shift(seed0 + k, 0), 0.5, seed=seed0 + k)
        for f in (f0, f1):
            bufs.append(torch.from_numpy(f).pin_memory())
    return bufs


def test_serve_stalled_producer_times_out_with_every_result(vtg_lib, ctx):
    sizes = [(640, 480), (1280, 720), (640, 480), (960, 544)]
    bufs = _frames(sizes, 80)
    streams = [dict(width=w, height=h, fps=100.0, start_s=0.0, frames=200) for w, h in sizes]
    lk = vtg_lib.config(64, 64, levels=4)
    st = vtg_lib.serve(ctx, streams, [b.data_ptr() for b in bufs], lk, duration_s=2.0, stall_at_s=0.3,
                       stall_timeout_s=0.2, allow_timeout=True)
    assert st["rc"] == vtg_lib.ETIMEOUT
    assert 0 < st["submitted"] < st["requests"]
    assert st["served"] + st["skipped"] == st["submitted"]  # everything handed over came back


def test_serve_refuses_malformed_stream_descriptions(vtg_lib, ctx):
    sizes = [(640, 480), (16, 16), (1280, 720), (640, 480)]
    bufs = _frames(sizes, 90)
    streams = [dict(width=640, height=480, fps=60.0, start_s=0.0, frames=10),
               dict(width=16, height=16, fps=60.0, start_s=0.0, frames=10),  # below the smallest picture
               dict(width=1280, height=720, fps=60.0, start_s=0.0, frames=10),
               dict(width=640, height=480, fps=0.0, start_s=0.0, frames=10)]  # no rate
    lk = vtg_lib.config(64, 64, levels=4)
    st = vtg_lib.serve(ctx, streams, [b.data_ptr() for b in bufs], lk, duration_s=1.0)
    assert st["streams_rejected"] == 2 and st["streams_admitted"] == 2
    assert st["requests"] == st["served"] == 20


def test_serve_live_under_overload_counts_skips(vtg_lib, ctx):
    """LIVE streams at a rate past what the GPU serves: frames queued behind a newer one are skipped and counted, so
    the latency of what is served stays bounded instead of a backlog growing."""
    sizes = [(1920, 1080)] * 6
    bufs = _frames(sizes, 95)
    streams = [dict(width=w, height=h, fps=3000.0, start_s=0.0, frames=300) for w, h in sizes]
    lk = vtg_lib.config(64, 64, levels=4)
    st = vtg_lib.serve(ctx, streams, [b.data_ptr() for b in bufs], lk, duration_s=2.0, live=True)
    assert st["skipped"] > 0
    assert st["served"] + st["skipped"] + st["dropped"] == st["requests"]
    ordered = vtg_lib.serve(ctx, streams, [b.data_ptr() for b in bufs], lk, duration_s=2.0, live=False)
    assert ordered["skipped"] == 0 and st["p99_ms"] < ordered["p99_ms"]


def test_server_search_request_matches_a_direct_search(vtg_lib, ctx):
    """A frame submitted with VTG_REQ_SEARCH comes back with the appearance search of its level 1 (step 2, the whole
    plane, the server's template): the same corner and score as vtg_search_run on that plane with that template."""
    import oracle as O

    seq = _seq(640, 480, 1, seed=140)
    frame = seq[1].numpy()
    level1 = O.pyramid(frame, 4)[1]
    app, norm = O.cut_template(level1.astype(np.float32), 150, 90, 32, 21)
    srv = vtg_lib.Server(ctx, vtg_lib.config(64, 64, levels=4))
    srv.template(app, norm)
    sid = srv.open(640, 480, seq[0].data_ptr())
    assert sid >= 0
    assert srv.submit(sid, seq[1].data_ptr(), flags=vtg_lib.REQ_SEARCH, tag=7) >= 0
    res = _drain(srv, 1)
    srv.close()
    assert len(res) == 1 and res[0]["status"] == vtg_lib.RES_DONE and res[0]["searched"] == 1
    got = res[0]["found"]
    t = vtg_lib.Tracker(ctx, vtg_lib.config(640, 480, levels=4))
    t.build(0, frame)
    t.sync()
    ptr, lw, lh, lp = vtg_lib.level_device(t, 0, 1)
    s = vtg_lib.Search(ctx, lw, lh, 32, 21)
    s.template(app, norm)
    want = s.run(ptr, lw, lh, lp, vtg_lib.PLANE_F32, 1, lw, 1, lh, 2, vtg_lib.NCC_F32)
    s.close()
    t.close()
    assert (got["hx"], got["hy"], got["ntop"], got["cells"]) == (want["hx"], want["hy"], want["ntop"], want["cells"])
    assert got["ncc"] == want["ncc"] and got["second"] == want["second"]
    assert (got["hx"], got["hy"]) == (300, 180)  # the template's own corner, in half pixels


def test_server_search_scratch_at_admission(vtg_lib, ctx):
    """With a template set, both slots' search scratch is charged to the budget when a stream is admitted, sized for the
    stream's level 1; a step that searches then allocates nothing (the loop never allocates inside a step)."""
    import ctypes

    seq = _seq(640, 480, 1, seed=141)
    app = np.zeros((21, 32), np.float32)
    app[::2] = 1.0
    app -= np.float32(app.mean(dtype=np.float64))
    norm = float((app.astype(np.float64) ** 2).sum())
    L = vtg_lib.lib()
    L.vtg_search_bytes.argtypes = [ctypes.c_int] * 4
    L.vtg_search_bytes.restype = ctypes.c_size_t
    srv = vtg_lib.Server(ctx, vtg_lib.config(64, 64, levels=4))
    srv.template(app, norm)
    used0 = ctx.used()
    sid = srv.open(640, 480, seq[0].data_ptr())
    assert sid >= 0
    tracker = L.vtg_tracker_bytes(ctypes.byref(vtg_lib.config(640, 480, levels=4)))
    scratch = L.vtg_search_bytes(320, 240, 32, 21)
    assert ctx.used() - used0 == tracker + 2 * scratch
    used1 = ctx.used()
    assert srv.submit(sid, seq[1].data_ptr(), flags=vtg_lib.REQ_SEARCH) >= 0
    res = _drain(srv, 1)
    assert len(res) == 1 and res[0]["status"] == vtg_lib.RES_DONE and res[0]["searched"] == 1
    assert ctx.used() == used1
    srv.close()
