"""Frame generation on the GPU (vtg_framegen) against the reference's framegen.c (tests/golden/framegen.npz) and the
oracle: every level's raw, filtered and upscaled field, the middle-instant field, the scene verdict, the generated
frame (Q6) and its bytes, all bit for bit (whole-number planes: every sum is exact)."""
import ctypes as C
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


def _run(vtg_lib, ctx, f0, f1):
    """(fields dict, frame Q6, bytes) of one generated frame on the GPU."""
    import torch

    h, w = f0.shape
    a, b = _dev(O.pyramid(f0, 1)[0]), _dev(O.pyramid(f1, 1)[0])
    out = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    pic = np.zeros((h, w), np.uint8)
    fg = vtg_lib.Framegen(ctx, w, h)
    vtg_lib.check(vtg_lib.lib().vtg_framegen_run(fg.h, a.data_ptr(), w, b.data_ptr(), w, out.data_ptr(), w,
                                                  pic.ctypes.data, vtg_lib.HOST, None), "vtg_framegen_run")
    fields = fg.fields()
    frame = out.cpu().numpy()
    fg.close()
    return fields, frame, pic


def _cases(g):
    for kind, (scene, w, h, sx, sy, seed) in zip(g["kinds"], g["cases"]):
        f0, f1 = S.framegen_pair("scene" if scene else "pair", int(w), int(h), (float(sx), float(sy)), int(seed))
        assert [O.fnv(f0), O.fnv(f1)] == [int(v) for v in g[str(kind) + "_frames_fnv"]]
        yield str(kind), f0, f1


def test_framegen_against_reference_fixture(vtg_lib, ctx, golden):
    g = np.load(os.path.join(golden, "framegen.npz"))
    for kind, f0, f1 in _cases(g):
        r, frame, pic = _run(vtg_lib, ctx, f0, f1)
        assert r["scene"] == int(g[kind + "_scene"]), kind
        for k in ("raw", "fil", "up"):
            got = np.concatenate([a.ravel() for a in r[k]])
            assert got.tobytes() == g[kind + "_" + k].tobytes(), (kind, k)
        assert r["mid"].ravel().tobytes() == g[kind + "_mid"].tobytes(), kind
        assert O.fnv(frame) == int(g[kind + "_out_fnv"]), kind
        assert O.fnv(pic) == int(g[kind + "_pic_fnv"]), kind


@pytest.mark.parametrize("w,h,shift,amp,seed", [(256, 192, (30.0, -22.0), 2.0, 5), (401, 257, (-1.2, 0.4), 0.0, 6),
                                                (130, 66, (4.5, 7.5), 1.0, 7), (1920, 1080, (-17.0, 12.0), 3.0, 8),
                                                (64, 64, (10.0, -7.0), 1.0, 9), (128, 96, (40.0, 30.0), 4.0, 10),
                                                (96, 200, (-45.0, 60.0), 0.0, 11)])
def test_framegen_against_oracle(vtg_lib, ctx, w, h, shift, amp, seed):
    f0, f1, _, _ = S.warp_pair(w, h, shift, amp, seed=seed)
    r, frame, pic = _run(vtg_lib, ctx, f0, f1)
    o = O.framegen(O.pyramid(f0, 1)[0], O.pyramid(f1, 1)[0])
    assert r["scene"] == o["scene"]
    for k in ("raw", "fil", "up"):
        for L, (a, b) in enumerate(zip(r[k], o[k])):
            assert a.tobytes() == b.tobytes(), (k, L)
    assert r["mid"].tobytes() == o["mid"].tobytes()
    assert np.array_equal(frame, o["out"]) and np.array_equal(pic, o["pic"])


@pytest.mark.parametrize("w,h", [(8192, 96), (96, 8192)])
def test_framegen_largest_sides(vtg_lib, ctx, w, h):
    """The widest and the tallest frames frame generation takes (8192 a side) against the oracle, bit for bit."""
    f0, f1, _, _ = S.warp_pair(w, h, (6.0, -3.5), 1.0, seed=w + h)
    r, frame, pic = _run(vtg_lib, ctx, f0, f1)
    o = O.framegen(O.pyramid(f0, 1)[0], O.pyramid(f1, 1)[0])
    assert r["scene"] == o["scene"]
    for k in ("raw", "fil", "up"):
        for L, (a, b) in enumerate(zip(r[k], o[k])):
            assert a.tobytes() == b.tobytes(), (k, L)
    assert r["mid"].tobytes() == o["mid"].tobytes()
    assert np.array_equal(frame, o["out"]) and np.array_equal(pic, o["pic"])


def test_framegen_api(vtg_lib, ctx):
    L = vtg_lib.lib()
    h = C.c_void_p()
    assert L.vtg_framegen_create(ctx.h, 63, 200, C.byref(h)) == vtg_lib.EINVAL  # the field needs two levels
    assert L.vtg_framegen_bytes(63, 200) == 0
    fg = vtg_lib.Framegen(ctx, 1920, 1080)
    assert fg.levels == 6 and fg.shapes[0] == (960, 540, 120, 68) and fg.shapes[-1] == (30, 17, 4, 3)
    a = _dev(np.zeros((1080, 1920), np.float32))
    assert L.vtg_framegen_run(fg.h, a.data_ptr(), 1919, a.data_ptr(), 1920, None, 0, None, vtg_lib.HOST,
                              None) == vtg_lib.EINVAL  # pitch < w
    assert L.vtg_framegen_fields(fg.h, 6, None, None, None, None, None, vtg_lib.HOST, None) == vtg_lib.EINVAL
    # two equal flat frames: no motion anywhere, the frame itself
    assert L.vtg_framegen_run(fg.h, a.data_ptr(), 1920, a.data_ptr(), 1920, None, 0, None, vtg_lib.HOST, None) == 0
    r = fg.fields()
    assert r["scene"] == 0 and not r["mid"]["x"].any() and not r["mid"]["y"].any()
    fg.close()
