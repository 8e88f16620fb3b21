"""store_appearance on the GPU (vtg_store_appearance): the appearance template cut from a tracker's resident pyramid.
Bar: validity, level, fraction, norm and the 32 x 21 template bit for bit against the reference (tests/golden/
appearance.npz) and the oracle; then the template, searched for on its own level, is found where it was cut."""
import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu


def test_appearance_against_reference_fixture(vtg_lib, ctx, golden):
    g = np.load(golden + "/appearance.npz")
    for i, (w, h, levels, seed) in enumerate(g["cases"]):
        w, h, levels = int(w), int(h), int(levels)
        f = S.build_frame("warp", w, h, int(seed))
        assert O.fnv(f) == int(g["case%d_frame_fnv" % i])
        t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=levels))
        t.build(1, f)
        for k, (cx, cy, rw, rh) in enumerate(g["case%d_regions" % i]):
            a = t.store_appearance(1, float(cx), float(cy), float(rw), float(rh))
            assert int(a["valid"]) == int(g["case%d_valid" % i][k]), (i, k)
            if a["valid"]:
                fx, fy, norm = g["case%d_f" % i][k]
                assert a["level"] == int(g["case%d_level" % i][k]) and (a["fx"], a["fy"]) == (fx, fy)
                assert np.float32(a["norm"]).tobytes() == norm.tobytes(), (i, k)
                assert O.fnv(a["pix"]) == int(g["case%d_pix_fnv" % i][k]), (i, k)
        t.close()


def test_appearance_against_oracle_device_outputs(vtg_lib, ctx):
    """Random regions of a stretched and smoothed 333 x 199 frame (3 levels); the template and norm also written to
    device memory, in one 673-float buffer and in two."""
    import ctypes as C

    import torch

    w, h, levels = 333, 199, 3
    f = S.build_frame("low", w, h, 3)
    t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=levels, cell_w=8, cell_h=8))
    t.set_build(vtg_lib.BUILD_CONTRAST | vtg_lib.BUILD_PRE_GAUSS)
    t.build(0, f)
    P = O.pyramid(f, levels, 3)
    L = vtg_lib.lib()
    one = torch.zeros(673, dtype=torch.float32, device="cuda")
    pix = torch.zeros(672, dtype=torch.float32, device="cuda")
    norm = torch.zeros(1, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    u = S.uniform(3, 600, 4 * 200).reshape(200, 4)
    regions = np.stack([u[:, 0] * w, u[:, 1] * h, 10 + u[:, 2] * w / 2, 10 + u[:, 3] * h / 2], 1).astype(np.float32)
    valid = 0
    for cx, cy, rw, rh in regions:
        a = t.store_appearance(0, float(cx), float(cy), float(rw), float(rh))
        o = O.store_appearance(P, float(cx), float(cy), float(rw), float(rh))
        assert a["valid"] == o["valid"]
        if not a["valid"]:
            continue
        valid += 1
        assert (a["level"], a["fx"], a["fy"]) == (o["level"], o["fx"], o["fy"])
        assert a["pix"].tobytes() == o["pix"].tobytes() and np.float32(a["norm"]).tobytes() == o["norm"].tobytes()
        info = vtg_lib.Appearance()
        vtg_lib.check(L.vtg_store_appearance(t.h, 0, float(cx), float(cy), float(rw), float(rh), one.data_ptr(),
                                             one.data_ptr() + 4 * 672, C.byref(info), vtg_lib.DEVICE, None), "app")
        vtg_lib.check(L.vtg_store_appearance(t.h, 0, float(cx), float(cy), float(rw), float(rh), pix.data_ptr(),
                                             norm.data_ptr(), C.byref(info), vtg_lib.DEVICE, None), "app")
        t.sync()
        got = one.cpu().numpy()
        assert got[:672].tobytes() == a["pix"].tobytes() and got[672] == a["norm"]
        assert pix.cpu().numpy().tobytes() == a["pix"].tobytes() and norm.cpu().numpy()[0] == a["norm"]
    assert valid > 50
    # out of range: no outputs needed, none written
    info = vtg_lib.Appearance()
    assert L.vtg_store_appearance(t.h, 0, 2.0, 2.0, 100.0, 100.0, None, None, C.byref(info), vtg_lib.HOST, None) == 0
    assert info.valid == 0
    assert L.vtg_store_appearance(t.h, 2, 100.0, 100.0, 100.0, 100.0, None, None, C.byref(info), vtg_lib.HOST,
                                  None) == vtg_lib.EINVAL
    t.close()


def test_appearance_found_by_search(vtg_lib, ctx):
    """The cut template, searched for over its level's resident plane (search_slot, F32), is found at the corner it
    was cut from with a score of 1."""
    w, h = 1280, 720
    f = S.build_frame("warp", w, h, 8)
    t = vtg_lib.Tracker(ctx, vtg_lib.config(w, h, levels=4))
    t.build(0, f)
    cx, cy, rw, rh = 611.0, 377.0, 140.0, 90.0
    a = t.store_appearance(0, cx, cy, rw, rh)
    assert a["valid"] and a["level"] == 2
    plane, lw, lh, lp = vtg_lib.level_device(t, 0, a["level"])
    s = vtg_lib.Search(ctx, lw, lh)
    s.template(a["pix"], float(a["norm"]))
    found = s.run(plane, lw, lh, lp, vtg_lib.PLANE_F32, 1, lw, 1, lh, 1, vtg_lib.NCC_F32)
    x0 = int(cx / 4) - 16
    y0 = int(cy / 4) - 10
    assert (found["hx"], found["hy"]) == (2 * x0, 2 * y0)
    assert abs(found["ncc"] - 1.0) < 1e-5
    s.close()
    t.close()
