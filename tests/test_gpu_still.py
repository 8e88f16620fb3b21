"""The still picture on the GPU (vtg_still): still_decide and still_update against the reference's own still.c
(tests/golden/still.npz) bit for bit, and the whole frame with the GPU's own vectors against the oracle.

- Fed the reference's vectors of each frame, the GPU's decision and update give the reference's still_hash on every
  frame: the cells' states (CHANGED, MOVING, the count), and the mean plane, bit for bit. The motion record matches:
  its counts exactly, its floats within 1e-6 relative (FP64 / double-double where the reference has long double).
- With its own vectors, the GPU's decision on those vectors equals the oracle's decision on the same vectors, and its
  mean equals the oracle's, bit for bit, every frame. Its vectors agree with the FP64 oracle's from the same mean
  within 0.01 px."""
import os

import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu

TOL_PX = 0.01
FLOATS = ("count_mean", "drift_u", "drift_v", "drift_rms", "diff_median", "diff_limit")
INTS = ("cols", "rows", "tracked", "moving", "frames")


def _dev(a):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    torch.cuda.synchronize()
    return t


def _motion_equal(got, want, k):
    for f in INTS:
        assert int(got[f]) == int(want[f]), (k, f, got[f], want[f])
    for f in FLOATS:
        assert np.isclose(float(got[f]), float(want[f]), rtol=1e-6, atol=1e-9), (k, f, got[f], want[f])


def test_still_decision_on_reference_cells(vtg_lib, ctx, golden):
    g = np.load(os.path.join(golden, "still.npz"))
    w, h, n, seed, jump = (int(v) for v in g["seq"])
    avg, px, grey = g["cfg"]
    frames = S.still_sequence(w, h, n, seed, jump_at=jump)
    assert [O.fnv(f) for f in frames] == [int(v) for v in g["frames_fnv"]]
    st = vtg_lib.Still(ctx, w, h, int(avg), float(px), float(grey))
    exact = 0
    for k, f in enumerate(frames):
        cur = _dev(O.pyramid(f, 1)[0])
        st.frame(cur.data_ptr(), w, cells=g["cells"][k])
        cells, m, mean = st.read()
        assert np.array_equal(cells["state"], g["cells"][k]["state"]), k
        assert O.still_hash(cells, mean) == int(g["hashes"][k]), k
        _motion_equal(m, g["motion"][k], k)
        exact += m.tobytes() == g["motion"][k].tobytes()
    assert exact >= len(frames) - 1  # floats equal to the bit but where one lies at a rounding boundary
    assert int(g["motion"]["moving"][jump]) == w // 16 * (h // 8)  # the fixture's frame where everything changed
    st.close()


@pytest.mark.parametrize("w,h,frames,avg,px,grey", [(320, 240, 12, 8, 1.0, 4.0), (640, 480, 6, 4, 0.5, 3.0),
                                                    (200, 121, 5, 16, 2.0, 6.0), (32, 32, 4, 1, 1.0, 4.0),
                                                    (47, 33, 6, 3, 0.0, 0.0)])
def test_still_gpu_vectors(vtg_lib, ctx, w, h, frames, avg, px, grey):
    seq = S.still_sequence(w, h, frames, seed=21, jump_at=frames - 2, mover=20)
    st = vtg_lib.Still(ctx, w, h, avg, px, grey)
    ref = O.Still(w, h, avg, px, grey)
    cfg = O.still_cfg()
    prev_mean = None
    for k, f in enumerate(seq):
        plane = O.pyramid(f, 1)[0]
        cur = _dev(plane)
        st.frame(cur.data_ptr(), w)
        cells, m, mean = st.read()
        # the decision and the update on the GPU's own vectors: the oracle's, bit for bit
        ocells, om = ref.frame(plane, cells=cells)
        assert np.array_equal(cells["state"], ocells["state"]), k
        assert np.array_equal(mean, ref.mean), k
        _motion_equal(m, om, k)
        if k == 0:
            assert not cells["u"].any() and not cells["v"].any()  # no vectors on the first frame
        else:
            # the GPU's vectors from the same mean against the FP64 oracle's
            out, fc = O.cells([prev_mean], [plane], 0, cfg, 16, 8, max_fb=O.STILL_FB, mode=O.F64, threads=8)
            lk_g, lk_o = cells["state"] & 0xff, fc["state"] & 0xff
            assert np.mean(lk_g == lk_o) >= 0.99, k
            both = (lk_g == 0) & (lk_o == 0)
            if both.any():  # after the brightness jump most patches fail their residual
                err = np.maximum(np.abs(cells["u"] - fc["u"]), np.abs(cells["v"] - fc["v"]))[both]
                assert err.max() < TOL_PX, (k, float(err.max()))
            # mean |frame - mean|: exact sums on the second frame (both planes whole numbers), float sums after it
            # (the mean is fractional), where the summation order moves the last bit
            assert np.allclose(cells["diff"], fc["diff"], rtol=1e-6, atol=1e-6), k
            if k == 1:
                assert np.array_equal(cells["diff"], fc["diff"])
        prev_mean = mean
    assert int(m["frames"]) == frames
    st.close()
    ref.close()


def test_still_api(vtg_lib, ctx):
    import ctypes as C

    import torch

    L = vtg_lib.lib()
    bad = vtg_lib.StillConfig(16, 240, 8, 1.0, 4.0)  # narrower than a patch's reach
    h = C.c_void_p()
    assert L.vtg_still_create(ctx.h, C.byref(bad), C.byref(h)) == vtg_lib.EINVAL
    assert L.vtg_still_bytes(C.byref(bad)) == 0
    st = vtg_lib.Still(ctx, 96, 64)
    plane = _dev(O.pyramid(S.noise_frame(96, 64, seed=3), 1)[0])
    assert L.vtg_still_frame(st.h, plane.data_ptr(), 95, None, vtg_lib.HOST, None) == vtg_lib.EINVAL  # pitch < w
    # the caller's cells from device memory, and the results read into device memory
    cells = np.zeros(6 * 8, vtg_lib.CELL_DTYPE)
    cells["state"] = 4  # every patch lost (LK_RESIDUAL): each cell's own evidence, so all changed and all moving
    dcells = torch.from_numpy(cells.view(np.uint8)).cuda()
    torch.cuda.synchronize()
    assert L.vtg_still_frame(st.h, plane.data_ptr(), 96, dcells.data_ptr(), vtg_lib.DEVICE, None) == 0
    out = torch.zeros(6 * 8 * 24, dtype=torch.uint8, device="cuda")
    assert L.vtg_still_read(st.h, out.data_ptr(), None, None, 0, vtg_lib.DEVICE, None) == 0
    L.vtg_ctx_sync(ctx.h, 5000)
    got = out.cpu().numpy().view(vtg_lib.CELL_DTYPE)
    assert np.all(got["state"] == (4 | 0x100 | 0x200 | (1 << 16)))
    p, pitch = C.c_void_p(), C.c_int()
    assert L.vtg_still_mean(st.h, C.byref(p), C.byref(pitch)) == 0 and pitch.value >= 96
    _, m, mean = st.read()
    assert np.array_equal(mean, plane.cpu().numpy())  # weight 1: the frame itself
    assert int(m["moving"]) == 48 and int(m["frames"]) == 1
    st.close()
