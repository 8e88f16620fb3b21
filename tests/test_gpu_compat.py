"""The reference's own kernel signatures (include/vtg_compat.h) on the GPU, called the way the reference's C code calls
its _vx kernels: planes in its padded layout (src/kern/plane.h), in host memory and in device memory, image kernels
over row ranges as a thread team splits them, LK one point at a time with a separate flowback call.

The padding of every input plane is NaN: a kernel that read it instead of clamping would return NaN. Results are held
to the same bars as the native API: pyramids bit-exact, flow within 0.01 px of the reference's lk_track_vx, the
correlation within 1e-5 of tk_correlate."""
import os

import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu

TOL_PX = 0.01
PAD_X, PAD_Y = 32, 4  # VT_PAD_X, VT_PAD_Y, src/kern/plane.h:14-15


@pytest.fixture(scope="module")
def torch_cuda():
    import torch

    return torch


class Plane:
    """A plane in the reference's layout: stride = round16(w) + 2 PAD_X floats, PAD_Y rows above and below."""

    def __init__(self, vtg, w, h, torch=None):
        self.w, self.h = w, h
        self.stride = ((w + 15) & ~15) + 2 * PAD_X
        buf = np.full((h + 2 * PAD_Y, self.stride), np.nan, np.float32)
        if torch is not None:
            self.buf = torch.from_numpy(buf).cuda()
            torch.cuda.synchronize()  # the adapter's stream does not wait for torch's
            base = self.buf.data_ptr()
        else:
            self.buf = buf
            base = buf.ctypes.data
        self.ref = vtg.RefPlane(base + 4 * (PAD_Y * self.stride + PAD_X), w, h, self.stride)

    def set(self, a):
        if isinstance(self.buf, np.ndarray):
            self.buf[PAD_Y:PAD_Y + self.h, PAD_X:PAD_X + self.w] = a
        else:
            import torch

            self.buf[PAD_Y:PAD_Y + self.h, PAD_X:PAD_X + self.w] = torch.from_numpy(np.ascontiguousarray(a)).cuda()
            torch.cuda.synchronize()

    def get(self):
        b = self.buf if isinstance(self.buf, np.ndarray) else self.buf.cpu().numpy()
        return b[PAD_Y:PAD_Y + self.h, PAD_X:PAD_X + self.w].copy()


def _pyramid(vtg, L, frame, levels, torch=None):
    """img_u8_to_q6 then img_reduce per level, each in two row halves (a team of two)."""
    h, w = frame.shape
    planes = [Plane(vtg, w, h, torch)]
    if torch is not None:
        src = torch.from_numpy(np.ascontiguousarray(frame)).cuda()
        torch.cuda.synchronize()
        sp = src.data_ptr()
    else:
        src = np.ascontiguousarray(frame)
        sp = src.ctypes.data
    for y0, y1 in ((0, h // 2), (h // 2, h)):
        L.img_u8_to_q6_cuda(planes[0].ref, sp, w, y0, y1)
        assert L.vtg_compat_error() == 0
    for lv in range(1, levels):
        sw, sh = planes[-1].w, planes[-1].h
        p = Plane(vtg, (sw + 1) // 2, (sh + 1) // 2, torch)
        for y0, y1 in ((0, p.h // 2), (p.h // 2, p.h)):
            L.img_reduce_cuda(p.ref, planes[-1].ref, y0, y1)
            assert L.vtg_compat_error() == 0
        planes.append(p)
    return planes, src


@pytest.mark.parametrize("w,h,levels,where", [(97, 61, 4, "host"), (640, 480, 3, "host"), (640, 480, 3, "device"),
                                              (1281, 719, 5, "device")])
def test_compat_pyramid(vtg_lib, torch_cuda, w, h, levels, where):
    L = vtg_lib.compat()
    frame = S.noise_frame(w, h, seed=w + h)
    planes, _ = _pyramid(vtg_lib, L, frame, levels, torch_cuda if where == "device" else None)
    ref = O.pyramid(frame, levels)
    for lv in range(levels):
        assert np.array_equal(planes[lv].get(), ref[lv]), lv


@pytest.mark.parametrize("where", ["host", "device"])
def test_compat_image_kernels_m1(vtg_lib, torch_cuda, golden, where):
    """img_norm / img_minmax / img_gauss5 / img_sobel / img_absdiff _cuda on the M1 gate's 640 x 480 frame, each over
    three row ranges as a team would split them, reproduce the gate's hash lines (logs/m1/host/m1-host-640x480.txt);
    then the stretch tk_build makes (vtg_contrast_gain's gain and offset) against the oracle."""
    import ctypes as C
    import json

    L = vtg_lib.compat()
    with open(os.path.join(golden, "m1_m2.json")) as f:
        m1 = json.load(f)["m1"]
    tc = torch_cuda if where == "device" else None
    w, h = 640, 480
    q = O.pyramid(O.m1_image(w, h), 1)[0]
    src = Plane(vtg_lib, w, h, tc)
    src.set(q)
    ranges = ((0, 100), (100, 333), (333, h))
    out = {k: Plane(vtg_lib, w, h, tc) for k in ("norm", "gauss5", "sobel_x", "sobel_y", "absdiff", "stretch")}
    go = (C.c_float * 2)(0.75, 512.0)
    for y0, y1 in ranges:
        L.img_norm_cuda(out["norm"].ref, src.ref, go, y0, y1)
        assert L.vtg_compat_error() == 0
        L.img_gauss5_cuda(out["gauss5"].ref, src.ref, y0, y1)
        assert L.vtg_compat_error() == 0
        L.img_sobel_cuda(out["sobel_x"].ref, out["sobel_y"].ref, src.ref, y0, y1)
        assert L.vtg_compat_error() == 0
    for y0, y1 in ranges:  # the binomial is complete before it is read
        L.img_absdiff_cuda(out["absdiff"].ref, src.ref, out["gauss5"].ref, y0, y1)
        assert L.vtg_compat_error() == 0
    for k in ("norm", "gauss5", "sobel_x", "sobel_y", "absdiff"):
        assert "%016x" % O.fnv(out[k].get()) == m1[k + " 640x480"], k
    mm = (C.c_float * 2)()
    L.img_minmax_cuda(src.ref, mm, 0, h)
    assert L.vtg_compat_error() == 0 and list(mm) == m1["minmax 640x480"]
    L.img_minmax_cuda(src.ref, mm, 100, 101)
    assert list(mm) == list(O.minmax(q[100:101]))
    g = vtg_lib.contrast_gain(int(m1["minmax 640x480"][0]), int(m1["minmax 640x480"][1]))
    L.img_norm_cuda(out["stretch"].ref, src.ref, g.ctypes.data, 0, h)
    assert out["stretch"].get().tobytes() == O.norm(q, float(g[0]), float(g[1])).tobytes()
    # refusals: sizes that differ, a missing second output, rows outside the plane
    small = Plane(vtg_lib, w // 2, h, tc)
    L.img_gauss5_cuda(small.ref, src.ref, 0, 10)
    assert L.vtg_compat_error() == vtg_lib.EINVAL
    L.img_sobel_cuda(out["sobel_x"].ref, None, src.ref, 0, 10)
    assert L.vtg_compat_error() == vtg_lib.EINVAL
    L.img_minmax_cuda(src.ref, mm, 0, h + 1)
    assert L.vtg_compat_error() == vtg_lib.EINVAL


def test_compat_lk_track_and_flowback(vtg_lib, torch_cuda, golden):
    """lk_track_cuda + lk_flowback_cuda at every 6th of the first configuration's 1,200 cells, host pyramids and
    device pyramids, against the reference's lk_track_vx + lk_flowback_vx (tests/golden/lk_640x480.npz)."""
    import ctypes as C

    L = vtg_lib.compat()
    g = np.load(os.path.join(golden, "lk_640x480.npz"))
    f0, f1, _, _ = S.warp_pair(640, 480, (1.7, -0.8), 0.5, seed=1)
    assert O.fnv(f0) == int(g["f0_fnv"]) and O.fnv(f1) == int(g["f1_fnv"])
    ref = g["vx"].view(O.LK_OUT)
    cfg = vtg_lib.RefLkCfg(21, 21, 10, 0.01, 0.1, 25.0, 0)
    sel = np.arange(0, 1200, 6)
    for where in ("host", "device"):
        tc = torch_cuda if where == "device" else None
        P0, _ = _pyramid(vtg_lib, L, f0, 3, tc)
        P1, _ = _pyramid(vtg_lib, L, f1, 3, tc)
        I = (vtg_lib.RefPlane * 3)(*[p.ref for p in P0])
        J = (vtg_lib.RefPlane * 3)(*[p.ref for p in P1])
        out = np.zeros(len(sel), O.LK_OUT)
        for k, i in enumerate(sel):
            x, y = float(g["xs"][i]), float(g["ys"][i])
            o = out[k:k + 1]
            L.lk_track_cuda(I, J, 2, C.byref(cfg), x, y, 0.0, 0.0, o.ctypes.data, None)
            assert L.vtg_compat_error() == 0
            L.lk_flowback_cuda(I, J, 2, C.byref(cfg), x, y, 0.5, o.ctypes.data, None)
            assert L.vtg_compat_error() == 0
        r = ref[sel]
        assert (out["status"] == r["status"]).mean() >= 0.98
        ok = (out["status"] == 0) & (r["status"] == 0)
        assert ok.sum() > 0.8 * len(sel)
        err = np.maximum(np.abs(out["x"] - r["x"]), np.abs(out["y"] - r["y"]))[ok]
        assert err.max() <= TOL_PX, (where, float(err.max()))


def test_compat_still_vectors(vtg_lib, golden):
    """still_vectors_cuda over the running mean and the new plane, against the reference's still_vectors."""
    L = vtg_lib.compat()
    g = np.load(os.path.join(golden, "still_vectors.npz"))
    f0, f1, _, _ = S.warp_pair(640, 480, (0.6, -0.3), 0.3, seed=5)
    mean, cur = Plane(vtg_lib, 640, 480), Plane(vtg_lib, 640, 480)
    mean.set(O.pyramid(f0, 1)[0])
    cur.set(O.pyramid(f1, 1)[0])
    cfg = vtg_lib.RefLkCfg(15, 15, 6, 0.01, 0.1, 16.0, 0)
    import ctypes as C

    cells = np.zeros(40 * 60, O.CELL)
    L.still_vectors_cuda(mean.ref, cur.ref, C.byref(cfg), 0.25, cells.ctypes.data, 1, 2)  # not tid 0: nothing
    assert not cells.view(np.uint8).any()
    L.still_vectors_cuda(mean.ref, cur.ref, C.byref(cfg), 0.25, cells.ctypes.data, 0, 2)
    assert L.vtg_compat_error() == 0
    ref = g["cells"].view(O.CELL)
    assert np.array_equal(cells["diff"], ref["diff"])
    assert (cells["state"] == ref["state"]).mean() >= 0.99
    ok = (cells["state"] == 0) & (ref["state"] == 0)
    assert np.maximum(np.abs(cells["u"] - ref["u"]), np.abs(cells["v"] - ref["v"]))[ok].max() <= TOL_PX


def test_compat_tk_correlate(vtg_lib, torch_cuda, golden):
    """tk_correlate_cuda at the fixture's corners, host and device planes, against the reference's tk_correlate."""
    L = vtg_lib.compat()
    g = np.load(os.path.join(golden, "ncc_32x21.npz"))
    plane = O.pyramid(S.noise_frame(640, 480, seed=9), 1)[0]
    app, norm = O.cut_template(plane, 300, 200, 32, 21)
    app = np.ascontiguousarray(app, np.float32)
    for where, count in (("host", 150), ("device", 150)):
        p = Plane(vtg_lib, 640, 480, torch_cuda if where == "device" else None)
        p.set(plane)
        got = np.array([float(L.tk_correlate_cuda(p.ref, app.ctypes.data, float(norm), int(x), int(y)))
                        for x, y in zip(g["cx"][:count], g["cy"][:count])])
        assert L.vtg_compat_error() == 0
        assert np.abs(got - g["corr"][:count]).max() < 1e-5, where
        # search_at's bounds: -1 outside the valid corners, without a GPU call
        assert float(L.tk_correlate_cuda(p.ref, app.ctypes.data, float(norm), 0, 5)) == -1.0
        assert float(L.tk_correlate_cuda(p.ref, app.ctypes.data, float(norm), 640 - 33, 5)) == -1.0


def test_compat_detect_run(vtg_lib, torch_cuda, golden):
    """detect_run_cuda as seed_at calls the detection (detect_begin, the three stages, detect_finish), on padded planes in
    host and device memory, against the reference's own detect.c outputs (tests/golden/detect.npz) and the oracle."""
    L = vtg_lib.compat()
    g = np.load(os.path.join(golden, "detect.npz"))
    d0, _, _, _ = S.warp_pair(640, 480, (1.7, -0.8), 0.5, seed=1)
    d0 = d0.copy()
    d0[300:420, 40:200] = 128
    plane = O.pyramid(d0, 1)[0]
    xs = np.zeros(512, np.float32)
    ys = np.zeros(512, np.float32)
    for where in ("host", "device"):
        p = Plane(vtg_lib, 640, 480, torch_cuda if where == "device" else None)
        p.set(plane)
        p0 = 0
        for k, (which, rx, ry, rw, rh, margin, mx, md, q) in enumerate(g["cases"]):
            m = int(g["counts"][k])
            if int(which) == 0:
                n = L.detect_run_cuda(p.ref, rx, ry, rw, rh, int(margin), int(mx), md, q, xs.ctypes.data,
                                      ys.ctypes.data)
                assert L.vtg_compat_error() == 0
                assert n == m and np.array_equal(xs[:n], g["xs"][p0:p0 + m]), (where, k)
                assert np.array_equal(ys[:n], g["ys"][p0:p0 + m]), (where, k)
            p0 += m
        # a seed_at box against the oracle, and a rectangle wholly inside the margin
        n = L.detect_run_cuda(p.ref, 120.5, 90.25, 384.0, 307.0, 12, 128, 8.0, 0.05, xs.ctypes.data, ys.ctypes.data)
        oxs, oys = O.detect(plane, 120.5, 90.25, 384, 307, 12, 128, 8.0, 0.05)
        assert n == len(oxs) and np.array_equal(xs[:n], oxs) and np.array_equal(ys[:n], oys)
        assert L.detect_run_cuda(p.ref, 630.0, 470.0, 50.0, 50.0, 12, 64, 4.0, 0.05, xs.ctypes.data,
                                 ys.ctypes.data) == 0
        assert L.vtg_compat_error() == 0
    # more corners than detect_finish keeps: refused, nothing found
    assert L.detect_run_cuda(p.ref, 0.0, 0.0, 640.0, 480.0, 12, 513, 4.0, 0.05, xs.ctypes.data, ys.ctypes.data) == 0
    assert L.vtg_compat_error() == vtg_lib.EINVAL


def test_compat_refusals(vtg_lib):
    """Arguments out of range: a status, the LK point marked lost, the image untouched; no kernel runs."""
    import ctypes as C

    L = vtg_lib.compat()
    assert L.lk_tile_bytes_cuda() == 64
    a, b = Plane(vtg_lib, 64, 64), Plane(vtg_lib, 20, 20)
    a.set(np.zeros((64, 64), np.float32))
    before = b.get()
    L.img_reduce_cuda(b.ref, a.ref, 0, 20)  # 20 x 20 is not the reduce of 64 x 64
    assert L.vtg_compat_error() == vtg_lib.EINVAL
    assert np.array_equal(b.get(), before, equal_nan=True)
    I = (vtg_lib.RefPlane * 1)(a.ref)
    wide = vtg_lib.RefLkCfg(41, 21, 10, 0.01, 0.1, 25.0, 0)  # wider than a warp's lanes
    o = np.zeros(1, O.LK_OUT)
    L.lk_track_cuda(I, I, 0, C.byref(wide), 32.0, 32.0, 0.0, 0.0, o.ctypes.data, None)
    assert L.vtg_compat_error() == vtg_lib.EINVAL
    assert o["status"][0] == 1 and o["x"][0] == 32.0
