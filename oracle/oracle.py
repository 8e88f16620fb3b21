"""oracle.py -- TEST INFRASTRUCTURE ONLY: ctypes access to the checker's two libraries.

* ``liboracle.so`` -- this project's CPU restatement of the reference's pyramid / LK / NCC path (vtg_oracle.c).
* ``_ref/libvtref.so`` -- the reference's own kernel sources with a small harness (ref_driver.c, ref_track_tu.c), built
  only where the reference tree is present; absent elsewhere (``ref_available()`` says which).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module, as the checker. The
library under test never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LANE, F64 = 0, 1
OK, OUT, LOWEIG, RESIDUAL, FLOWBACK = 0, 1, 2, 4, 8
MAX_LEVELS = 8

# struct lk_out (src/kern/lk.h:33-40) / struct vt_cell (src/common/vt_proto.h:395-402) as numpy records.
LK_OUT = np.dtype([("x", "<f4"), ("y", "<f4"), ("min_eig", "<f4"), ("residual", "<f4"), ("cov_xx", "<f4"),
                   ("cov_xy", "<f4"), ("cov_yy", "<f4"), ("iters", "<u2"), ("status", "<u2")])
CELL = np.dtype([("u", "<f4"), ("v", "<f4"), ("diff", "<f4"), ("state", "<u4"), ("sigma", "<f4"), ("pad", "<f4")])
# What still_motion fills (src/kern/still.c:262-275), as the library's struct vtg_still_motion: 48 bytes.
STILL_MOTION = np.dtype([("cols", "<u4"), ("rows", "<u4"), ("tracked", "<u4"), ("moving", "<u4"),
                         ("count_mean", "<f4"), ("drift_u", "<f4"), ("drift_v", "<f4"), ("drift_rms", "<f4"),
                         ("diff_median", "<f4"), ("diff_limit", "<f4"), ("frames", "<u8")])
assert LK_OUT.itemsize == 32 and CELL.itemsize == 24


class Pyr(C.Structure):
    _fields_ = [("levels", C.c_int), ("w", C.c_int * MAX_LEVELS), ("h", C.c_int * MAX_LEVELS),
                ("stride", C.c_int * MAX_LEVELS), ("lv", C.c_void_p * MAX_LEVELS)]


class LkCfg(C.Structure):
    _fields_ = [("w", C.c_int), ("h", C.c_int), ("max_iter", C.c_int), ("eps", C.c_float),
                ("min_eig", C.c_float), ("max_residual", C.c_float)]


class Img(C.Structure):
    _fields_ = [("p", C.c_void_p), ("w", C.c_int), ("h", C.c_int), ("stride", C.c_int)]


class Found(C.Structure):
    _fields_ = [("hx", C.c_int), ("hy", C.c_int), ("ncc", C.c_double), ("second", C.c_double),
                ("ox", C.c_double), ("oy", C.c_double)]


def _build(target: str = "all") -> None:
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


_lib = None
_ref = None


def lib() -> C.CDLL:
    """liboracle.so, built on first use."""
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        src = os.path.join(HERE, "vtg_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            _build("all")
        _lib = C.CDLL(path)
        _lib.or_fnv.restype = C.c_uint64
        _lib.or_fnv.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        for name in ("or_ncc_at", "or_ncc_half"):
            f = getattr(_lib, name)
            f.restype = C.c_double
            f.argtypes = [C.POINTER(Img), C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int]
        _lib.or_peak_offset.restype = C.c_double
        _lib.or_peak_offset.argtypes = [C.c_double] * 3
        _lib.or_lk_track.argtypes = [C.POINTER(Pyr), C.POINTER(Pyr), C.c_int, C.POINTER(LkCfg), C.c_float, C.c_float,
                                     C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_int]
        _lib.or_lk_points.argtypes = [C.POINTER(Pyr), C.POINTER(Pyr), C.c_int, C.POINTER(LkCfg), C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_int, C.c_int]
        _lib.or_cells.argtypes = [C.POINTER(Pyr), C.POINTER(Pyr), C.c_int, C.POINTER(LkCfg), C.c_int, C.c_int,
                                  C.c_float, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        _lib.or_search_slot.argtypes = [C.POINTER(Img), C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                        C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(Found), C.c_void_p, C.c_void_p,
                                        C.c_void_p]
        _lib.or_ncc_map.argtypes = [C.POINTER(Img), C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
        _lib.or_cut_template.argtypes = [C.POINTER(Img), C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        _lib.or_u8_to_q6.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
        _lib.or_reduce.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
        _lib.or_minmax.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        _lib.or_norm.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        _lib.or_gauss5.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
        _lib.or_sobel.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        _lib.or_absdiff.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
        _lib.or_contrast_gain.argtypes = [C.c_int, C.c_int, C.c_void_p]
        _lib.or_build_input.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
        _lib.or_store_appearance.argtypes = [C.POINTER(Pyr), C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p,
                                             C.c_void_p]
        _lib.or_m1_image.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        _lib.or_m2_render.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        _lib.or_cell_centre.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(LkCfg), C.c_int, C.c_int,
                                        C.c_void_p, C.c_void_p]
        _lib.or_detect_geometry.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                            C.POINTER(DetGeo)]
        _lib.or_detect_maps.argtypes = [C.POINTER(Img), C.POINTER(DetGeo), C.c_void_p, C.c_void_p]
        _lib.or_detect_finish.argtypes = [C.POINTER(DetGeo), C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_float,
                                          C.c_void_p, C.c_void_p]
        _lib.or_still_create.restype = C.c_void_p
        _lib.or_still_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float]
        _lib.or_still_destroy.argtypes = [C.c_void_p]
        _lib.or_still_first.argtypes = [C.c_void_p]
        _lib.or_still_decide.argtypes = [C.c_void_p, C.c_void_p]
        _lib.or_still_update.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        _lib.or_still_finish.argtypes = [C.c_void_p]
        _lib.or_still_motion.argtypes = [C.c_void_p, C.c_void_p]
        _lib.or_fg_levels.argtypes = [C.c_int, C.c_int]
        _lib.or_framegen.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return _lib


class DetGeo(C.Structure):
    """struct or_det_geo: a detection region as detect_begin lays it out."""
    _fields_ = [(k, C.c_int) for k in ("x0", "y0", "x1", "y1", "ax", "cols", "rows", "nv", "cell_rows")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def detect_geometry(w, h, rx, ry, rw, rh, margin):
    """detect_begin's layout (src/kern/detect.c:28-66), or None when the rectangle is empty."""
    g = DetGeo()
    return g if lib().or_detect_geometry(w, h, rx, ry, rw, rh, margin, C.byref(g)) else None


def detect_maps(plane, g: DetGeo):
    """(resp rows x cols, cells cell_rows x nv): the Harris response and each cell's strongest (detect.c:68-141)."""
    plane = np.ascontiguousarray(plane, np.float32)
    m = img(plane)
    resp = np.zeros((g.rows, g.cols), np.float32)
    cell = np.zeros((g.cell_rows, g.nv), np.float32)
    lib().or_detect_maps(C.byref(m), C.byref(g), _p(resp), _p(cell))
    return resp, cell


def detect(plane, rx, ry, rw, rh, margin, max_n, min_dist, quality):
    """Corner detection as the tracker seeds features (track.c:988-992): (xs, ys), best first."""
    h, w = plane.shape
    g = detect_geometry(w, h, rx, ry, rw, rh, margin)
    if g is None:
        return np.zeros(0, np.float32), np.zeros(0, np.float32)
    resp, cell = detect_maps(plane, g)
    xs = np.zeros(max(max_n, 1), np.float32)
    ys = np.zeros(max(max_n, 1), np.float32)
    n = lib().or_detect_finish(C.byref(g), _p(resp), _p(cell), max_n, min_dist, quality, _p(xs), _p(ys))
    return xs[:n].copy(), ys[:n].copy()


def ref_detect(plane, rx, ry, rw, rh, margin, max_n, min_dist, quality):
    """The reference's own detection: (geometry dict, resp, cells, xs, ys), or None when the rectangle is empty."""
    plane = np.ascontiguousarray(plane, np.float32)
    h, w = plane.shape
    geo = np.zeros(9, np.int32)
    resp = np.zeros(w * h + 16 * w, np.float32)
    cell = np.zeros(w * h // 16 + 1024, np.float32)
    xs = np.zeros(max(max_n, 1), np.float32)
    ys = np.zeros(max(max_n, 1), np.float32)
    n = ref().ref_detect(_p(plane), w, h, rx, ry, rw, rh, margin, max_n, min_dist, quality, _p(geo), _p(resp),
                         _p(cell), _p(xs), _p(ys))
    if n < 0:
        return None
    g = dict(zip(("x0", "y0", "x1", "y1", "ax", "cols", "rows", "nv", "cell_rows"), [int(v) for v in geo]))
    return (g, resp[:g["rows"] * g["cols"]].reshape(g["rows"], g["cols"]).copy(),
            cell[:g["cell_rows"] * g["nv"]].reshape(g["cell_rows"], g["nv"]).copy(), xs[:n].copy(), ys[:n].copy())


def ref_available() -> bool:
    """True where oracle/_ref/libvtref.so, the reference's own kernels, is built or can be: where the reference tree the
    Makefile reads is on this host. Elsewhere the Makefile's `ref` target fails and the checks that need it are
    skipped."""
    path = os.path.join(HERE, "_ref", "libvtref.so")
    if os.path.exists(path):
        return True
    r = subprocess.run(["make", "-s", "-C", HERE, "ref"], capture_output=True)
    return r.returncode == 0 and os.path.exists(path)


def ref() -> C.CDLL:
    """oracle/_ref/libvtref.so: the reference's own code."""
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("oracle/_ref is not built: the reference sources are not on this machine")
        _ref = C.CDLL(os.path.join(HERE, "_ref", "libvtref.so"))
        _ref.ref_correlate.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
        _ref.ref_search_slot.restype = C.c_int
        _ref.ref_search_slot.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_float, C.c_int,
                                         C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_int]
        _ref.ref_search_half.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_float, C.c_int, C.c_void_p,
                                         C.c_void_p, C.c_void_p]
        _ref.ref_peak_offset.restype = C.c_double
        _ref.ref_detect.restype = C.c_int
        _ref.ref_detect.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                    C.c_int, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p]
        _ref.ref_peak_offset.argtypes = [C.c_double] * 3
        _ref.ref_lk_points.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        _ref.ref_pyramid.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        _ref.ref_tk_build.restype = C.c_int
        _ref.ref_store_appearance.restype = C.c_int
        _ref.ref_store_appearance.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                              C.c_float, C.c_void_p, C.c_void_p]
        _ref.ref_tk_build.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        _ref.ref_still_vectors.restype = C.c_int
        _ref.ref_still_vectors.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        _ref.ref_still_run.restype = C.c_int
        _ref.ref_framegen.restype = C.c_int
        _ref.ref_framegen.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _ref.ref_still_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return _ref


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def fnv(data: bytes | np.ndarray, h: int = 0xcbf29ce484222325) -> int:
    a = np.ascontiguousarray(data)
    return lib().or_fnv(h, a.ctypes.data, a.nbytes)


def level_dims(w: int, h: int, levels: int):
    dims = []
    for _ in range(levels):
        dims.append((w, h))
        w, h = (w + 1) // 2, (h + 1) // 2
    return dims


BUILD_CONTRAST = 1
BUILD_PRE_GAUSS = 2


def pyramid(frame: np.ndarray, levels: int, opts: int = 0):
    """The Q6 pyramid of a uint8 frame: a list of float32 planes (exact whole numbers), level 0 first. opts: tk_build's
    optional input steps, BUILD_CONTRAST and / or BUILD_PRE_GAUSS (src/kern/track.c:600-622)."""
    L = lib()
    frame = np.ascontiguousarray(frame, dtype=np.uint8)
    h, w = frame.shape
    out = []
    q = np.empty((h, w), np.float32)
    if opts:
        L.or_build_input(_p(frame), w, w, h, int(opts), _p(q), w)
    else:
        L.or_u8_to_q6(_p(frame), C.c_int(w), C.c_int(w), C.c_int(h), _p(q), C.c_int(w))
    out.append(q)
    for _ in range(1, levels):
        ph, pw = out[-1].shape
        d = np.empty(((ph + 1) // 2, (pw + 1) // 2), np.float32)
        L.or_reduce(_p(out[-1]), C.c_int(pw), C.c_int(ph), C.c_int(pw), _p(d), C.c_int(d.shape[1]))
        out.append(d)
    return out


def _plane(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    assert a.ndim == 2
    return a


def minmax(plane: np.ndarray):
    """img_minmax: (min, max) of a plane."""
    a = _plane(plane)
    out = np.zeros(2, np.float32)
    lib().or_minmax(_p(a), a.shape[1], a.shape[0], a.shape[1], _p(out))
    return float(out[0]), float(out[1])


def norm(plane: np.ndarray, gain: float, offset: float) -> np.ndarray:
    """img_norm: clamp(rint(plane x gain + offset), 0, 16320)."""
    a = _plane(plane)
    go = np.array([gain, offset], np.float32)
    d = np.empty_like(a)
    lib().or_norm(_p(a), a.shape[1], a.shape[0], a.shape[1], _p(go), _p(d), a.shape[1])
    return d


def gauss5(plane: np.ndarray) -> np.ndarray:
    """img_gauss5: the 5 x 5 binomial at every pixel."""
    a = _plane(plane)
    d = np.empty_like(a)
    lib().or_gauss5(_p(a), a.shape[1], a.shape[0], a.shape[1], _p(d), a.shape[1])
    return d


def sobel(plane: np.ndarray):
    """img_sobel: (ix, iy)."""
    a = _plane(plane)
    ix, iy = np.empty_like(a), np.empty_like(a)
    lib().or_sobel(_p(a), a.shape[1], a.shape[0], a.shape[1], _p(ix), _p(iy), a.shape[1])
    return ix, iy


def absdiff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """img_absdiff: |a - b|."""
    a, b = _plane(a), _plane(b)
    assert a.shape == b.shape
    d = np.empty_like(a)
    lib().or_absdiff(_p(a), _p(b), a.shape[1], a.shape[0], a.shape[1], _p(d), a.shape[1])
    return d


def contrast_gain(lo: int, hi: int):
    """tk_build's stretch gain and offset (float32) for Q6 minimum lo and maximum hi."""
    go = np.zeros(2, np.float32)
    lib().or_contrast_gain(int(lo), int(hi), _p(go))
    return go


def ref_tk_build(frame: np.ndarray, levels: int, opts: int = 0, x87: bool = False):
    """The reference's own tk_build of one frame (width a multiple of 16): its pyramid's planes, level 0 first."""
    frame = np.ascontiguousarray(frame, dtype=np.uint8)
    h, w = frame.shape
    dims = level_dims(w, h, levels)
    out = np.zeros(sum(a * b for a, b in dims), np.float32)
    rc = ref().ref_tk_build(_p(frame), w, h, levels, int(bool(opts & BUILD_CONTRAST)),
                            int(bool(opts & BUILD_PRE_GAUSS)), int(x87), _p(out))
    assert rc == 0, "tk_create refused the configuration"
    planes, off = [], 0
    for (lw, lh) in dims:
        planes.append(out[off:off + lw * lh].reshape(lh, lw))
        off += lw * lh
    return planes


APP_W, APP_H = 32, 21


def _app_result(pix, info):
    return {"pix": pix, "norm": np.float32(info[0]), "fx": np.float32(info[1]), "fy": np.float32(info[2]),
            "level": int(info[3]), "valid": bool(info[4])}


def store_appearance(levels_list, cx: float, cy: float, rw: float, rh: float) -> dict:
    """store_appearance on a pyramid (list of planes): pix (21 x 32 float32), norm, fx, fy, level, valid."""
    p = make_pyr(levels_list)
    pix = np.zeros((APP_H, APP_W), np.float32)
    info = np.zeros(5, np.float32)
    lib().or_store_appearance(C.byref(p), cx, cy, rw, rh, _p(pix), _p(info))
    return _app_result(pix, info)


def ref_store_appearance(frame: np.ndarray, levels: int, cx: float, cy: float, rw: float, rh: float) -> dict:
    """The reference's own store_appearance on the pyramid its tk_build makes of `frame` (width a multiple of 16)."""
    frame = np.ascontiguousarray(frame, dtype=np.uint8)
    h, w = frame.shape
    pix = np.zeros((APP_H, APP_W), np.float32)
    info = np.zeros(5, np.float32)
    assert ref().ref_store_appearance(_p(frame), w, h, levels, cx, cy, rw, rh, _p(pix), _p(info)) == 0
    return _app_result(pix, info)


def make_pyr(levels_list) -> Pyr:
    p = Pyr()
    p.levels = len(levels_list)
    for i, pl in enumerate(levels_list):
        assert pl.dtype == np.float32 and pl.flags.c_contiguous
        p.h[i], p.w[i] = pl.shape
        p.stride[i] = pl.shape[1]
        p.lv[i] = pl.ctypes.data
    p._keep = levels_list  # keeps the planes alive with the struct
    return p


def lk_cfg(w=21, h=21, max_iter=10, eps=0.01, min_eig=0.1, max_residual=25.0) -> LkCfg:
    return LkCfg(w, h, max_iter, eps, min_eig, max_residual)


def lk_points(I, J, top, cfg: LkCfg, xs, ys, gxs=None, gys=None, max_fb=0.0, mode=LANE, threads=1) -> np.ndarray:
    xs = np.ascontiguousarray(xs, np.float32)
    ys = np.ascontiguousarray(ys, np.float32)
    gxs = None if gxs is None else np.ascontiguousarray(gxs, np.float32)
    gys = None if gys is None else np.ascontiguousarray(gys, np.float32)
    out = np.zeros(len(xs), LK_OUT)
    pi, pj = make_pyr(I), make_pyr(J)
    lib().or_lk_points(C.byref(pi), C.byref(pj), top, C.byref(cfg), len(xs), _p(xs), _p(ys), _p(gxs), _p(gys),
                       C.c_float(max_fb), _p(out), mode, threads)
    return out


def grid_shape(w: int, h: int, cell_w: int, cell_h: int):
    return (h + cell_h - 1) // cell_h, (w + cell_w - 1) // cell_w


def cells(I, J, top, cfg: LkCfg, cell_w, cell_h, max_fb=0.0, mode=LANE, threads=1):
    """The per-cell grid over level 0 of I / J: (lk_out records, vt_cell records), row-major."""
    rows, cols = grid_shape(I[0].shape[1], I[0].shape[0], cell_w, cell_h)
    out = np.zeros(rows * cols, LK_OUT)
    cl = np.zeros(rows * cols, CELL)
    pi, pj = make_pyr(I), make_pyr(J)
    lib().or_cells(C.byref(pi), C.byref(pj), top, C.byref(cfg), cell_w, cell_h, C.c_float(max_fb), _p(out), _p(cl),
                   mode, threads)
    return out, cl


def cell_centres(w, h, cell_w, cell_h, pw=21, ph=21):
    """Cell centres as the per-cell grid places them (src/kern/still.c:127-130, margin = patch / 2 + 2)."""
    rows, cols = grid_shape(w, h, cell_w, cell_h)
    mx, my = float(pw // 2 + 2), float(ph // 2 + 2)
    c = np.arange(cols, dtype=np.float32) * cell_w + cell_w // 2
    r = np.arange(rows, dtype=np.float32) * cell_h + cell_h // 2
    c = np.clip(c, mx, np.float32(w - 1 - mx))
    r = np.clip(r, my, np.float32(h - 1 - my))
    xs, ys = np.meshgrid(c, r)
    return xs.astype(np.float32).ravel(), ys.astype(np.float32).ravel()


def img(plane: np.ndarray) -> Img:
    plane = np.ascontiguousarray(plane, np.float32)
    m = Img(plane.ctypes.data, plane.shape[1], plane.shape[0], plane.shape[1])
    m._keep = plane
    return m


def cut_template(plane, x0, y0, tw, th):
    app = np.empty(tw * th, np.float32)
    norm = np.zeros(1, np.float32)
    m = img(plane)
    lib().or_cut_template(C.byref(m), x0, y0, tw, th, _p(app), _p(norm))
    return app.reshape(th, tw), float(norm[0])


def ncc_at(plane, app, norm, x, y, mode=LANE) -> float:
    app = np.ascontiguousarray(app, np.float32)
    m = img(plane)
    return lib().or_ncc_at(C.byref(m), _p(app), app.shape[1], app.shape[0], norm, x, y, mode)


def ncc_half(plane, app, norm, hx, hy, mode=LANE) -> float:
    app = np.ascontiguousarray(app, np.float32)
    m = img(plane)
    return lib().or_ncc_half(C.byref(m), _p(app), app.shape[1], app.shape[0], norm, hx, hy, mode)


def ncc_map(plane, app, norm, x0, x1, y0, y1, mode=F64) -> np.ndarray:
    app = np.ascontiguousarray(app, np.float32)
    out = np.empty((y1 - y0 + 1, x1 - x0 + 1), np.float32)
    m = img(plane)
    lib().or_ncc_map(C.byref(m), _p(app), app.shape[1], app.shape[0], norm, x0, x1, y0, y1, mode, _p(out), 1)
    return out


def search_slot(plane, app, norm, x0, x1, y0, y1, step, mode=LANE):
    """search_slot: (found dict, per-cell map values, map x, map y)."""
    app = np.ascontiguousarray(app, np.float32)
    m = img(plane)
    h, w = plane.shape
    ncells = (w // 16 + 2) * (h // 16 + 2)
    mv = np.zeros(ncells, np.float32)
    mx = np.zeros(ncells, np.int32)
    my = np.zeros(ncells, np.int32)
    f = Found()
    lib().or_search_slot(C.byref(m), _p(app), app.shape[1], app.shape[0], norm, x0, x1, y0, y1, step, mode,
                         C.byref(f), _p(mv), _p(mx), _p(my))
    return {"hx": f.hx, "hy": f.hy, "ncc": f.ncc, "second": f.second, "ox": f.ox, "oy": f.oy}, mv, mx, my


def peak_offset(l, c, r) -> float:
    return lib().or_peak_offset(l, c, r)


def m1_image(w: int, h: int) -> np.ndarray:
    stride = (w + 15) & ~15
    a = np.zeros((h, stride), np.uint8)
    lib().or_m1_image(_p(a), w, h, stride)
    return a[:, :w].copy()


def m2_render(w: int, h: int, ox: int, oy: int) -> np.ndarray:
    a = np.zeros((h, w), np.uint8)
    lib().or_m2_render(_p(a), w, h, w, ox, oy)
    return a


# ---------------------------------------------------------------- the reference itself (oracle/_ref)

def ref_pyramid(frame: np.ndarray, levels: int, use_ref: bool = False):
    frame = np.ascontiguousarray(frame, np.uint8)
    h, w = frame.shape
    stride = (w + 15) & ~15
    buf = np.zeros((h, stride), np.uint8)
    buf[:, :w] = frame
    dims = level_dims(w, h, levels)
    out = np.zeros(sum(a * b for a, b in dims), np.float32)
    ref().ref_pyramid(_p(buf), stride, w, h, levels, int(use_ref), _p(out))
    planes, off = [], 0
    for (lw, lh) in dims:
        planes.append(out[off:off + lw * lh].reshape(lh, lw))
        off += lw * lh
    return planes


def ref_lk_points(f0, f1, levels, top, cfg: LkCfg, xs, ys, gxs=None, gys=None, max_fb=0.0, use_ref=False,
                  threads=8, base=0) -> np.ndarray:
    h, w = f0.shape
    stride = (w + 15) & ~15
    b0 = np.zeros((h, stride), np.uint8)
    b1 = np.zeros((h, stride), np.uint8)
    b0[:, :w] = f0
    b1[:, :w] = f1
    xs = np.ascontiguousarray(xs, np.float32)
    ys = np.ascontiguousarray(ys, np.float32)
    gxs = None if gxs is None else np.ascontiguousarray(gxs, np.float32)
    gys = None if gys is None else np.ascontiguousarray(gys, np.float32)
    out = np.zeros(len(xs), LK_OUT)
    ref().ref_lk_points(_p(b0), _p(b1), stride, w, h, levels, base, top, cfg.w, cfg.h, cfg.max_iter, C.c_float(cfg.eps),
                        C.c_float(cfg.min_eig), C.c_float(cfg.max_residual), C.c_float(max_fb), len(xs), _p(xs),
                        _p(ys), _p(gxs), _p(gys), int(use_ref), threads, _p(out))
    return out


def ref_still_vectors(f0, f1) -> np.ndarray:
    h, w = f0.shape
    stride = (w + 15) & ~15
    b0 = np.zeros((h, stride), np.uint8)
    b1 = np.zeros((h, stride), np.uint8)
    b0[:, :w] = f0
    b1[:, :w] = f1
    n = ((w + 15) // 16) * ((h + 7) // 8)
    out = np.zeros(n, CELL)
    got = ref().ref_still_vectors(_p(b0), _p(b1), stride, w, h, _p(out))
    assert got == n
    return out


def ref_correlate(plane, app, norm, xs, ys) -> np.ndarray:
    plane = np.ascontiguousarray(plane, np.float32)
    app = np.ascontiguousarray(app, np.float32)
    assert app.shape == (21, 32)
    xs = np.ascontiguousarray(xs, np.int32)
    ys = np.ascontiguousarray(ys, np.int32)
    out = np.zeros(len(xs), np.float64)
    ref().ref_correlate(_p(plane), plane.shape[1], plane.shape[0], _p(app), norm, len(xs), _p(xs), _p(ys), _p(out))
    return out


def ref_search_slot(plane, app, norm, x0, x1, y0, y1, step, level=0):
    plane = np.ascontiguousarray(plane, np.float32)
    app = np.ascontiguousarray(app, np.float32)
    h, w = plane.shape
    maxc = (w // 16 + 2) * (h // 16 + 2)
    mv = np.zeros(maxc, np.float32)
    mx = np.zeros(maxc, np.int32)
    my = np.zeros(maxc, np.int32)
    hx, hy = C.c_int(), C.c_int()
    ncc, second = C.c_double(), C.c_double()
    n = ref().ref_search_slot(_p(plane), w, h, level, _p(app), C.c_float(norm), x0, x1, y0, y1, step, C.byref(hx),
                              C.byref(hy), C.byref(ncc), C.byref(second), _p(mv), _p(mx), _p(my), maxc)
    if n < 0:
        raise RuntimeError("ref_search_slot: tracker set-up failed")
    return {"hx": hx.value, "hy": hy.value, "ncc": ncc.value, "second": second.value}, mv[:n], mx[:n], my[:n]


def ref_search_half(plane, app, norm, hxs, hys) -> np.ndarray:
    plane = np.ascontiguousarray(plane, np.float32)
    app = np.ascontiguousarray(app, np.float32)
    hxs = np.ascontiguousarray(hxs, np.int32)
    hys = np.ascontiguousarray(hys, np.int32)
    out = np.zeros(len(hxs), np.float64)
    ref().ref_search_half(_p(plane), plane.shape[1], plane.shape[0], _p(app), C.c_float(norm), len(hxs), _p(hxs),
                          _p(hys), _p(out))
    return out


# ---------------------------------------------------------------- the still picture (src/kern/still.c)

def still_cfg() -> LkCfg:
    """still.c's LK: a 15 x 15 patch, 6 iterations, eps 0.01, min_eig 0.1, residual 16 (src/kern/still.c:14-19)."""
    return lk_cfg(15, 15, 6, 0.01, 0.1, 16.0)


STILL_FB = 0.25  # FB_MAX, src/kern/still.c:19


class Still:
    """One camera's still picture, as the reference runs a frame: still_vectors unless it is the first frame (the
    per-cell grid from the mean to the frame, one level, OR_LANE by default), still_decide, still_update, still_finish.
    ``frame(cur, cells=...)`` takes the frame's vectors from the caller instead (their LK byte of state is what the
    decision reads)."""

    def __init__(self, w, h, avg=8, motion_px=1.0, motion_grey=4.0):
        self.w, self.h = w, h
        self.cols, self.rows = (w + 15) // 16, (h + 7) // 8
        self.s = lib().or_still_create(w, h, avg, C.c_float(motion_px), C.c_float(motion_grey))
        self.mean = np.zeros((h, w), np.float32)
        self.cells = np.zeros(self.cols * self.rows, CELL)

    def frame(self, cur, cells=None, mode=LANE, threads=1):
        """One frame on the Q6 plane cur (h x w): the cells after the decision and the motion record."""
        cur = np.ascontiguousarray(cur, np.float32)
        if cells is not None:
            self.cells = np.ascontiguousarray(cells, CELL).copy()
        elif not lib().or_still_first(self.s):
            _, self.cells = globals()["cells"]([self.mean], [cur], 0, still_cfg(), 16, 8, max_fb=STILL_FB, mode=mode,
                                               threads=threads)
        lib().or_still_decide(self.s, _p(self.cells))
        lib().or_still_update(self.s, _p(self.mean), self.w, _p(cur), self.w)
        lib().or_still_finish(self.s)
        m = np.zeros(1, STILL_MOTION)
        lib().or_still_motion(self.s, _p(m))
        return self.cells.copy(), m[0]

    def close(self):
        if self.s:
            lib().or_still_destroy(self.s)
            self.s = None

    def __del__(self):
        self.close()


def still_hash(cells: np.ndarray, mean: np.ndarray, h: int = 0xcbf29ce484222325) -> int:
    """still_hash (src/kern/still.c:253-259): the cells' bytes, then the mean's rows."""
    h = fnv(np.ascontiguousarray(cells, CELL), h)
    return fnv(np.ascontiguousarray(mean, np.float32), h)


def ref_still_run(frames, avg=8, motion_px=1.0, motion_grey=4.0):
    """The reference's still picture over 8-bit frames (src/host/m3_ref.c:272-283): per frame (cells, motion, hash),
    and the mean after the last frame."""
    f0 = np.ascontiguousarray(frames[0])
    h, w = f0.shape
    stride = (w + 15) & ~15
    buf = np.zeros((len(frames), h, stride), np.uint8)
    for k, f in enumerate(frames):
        buf[k, :, :w] = f
    n = ((w + 15) // 16) * ((h + 7) // 8)
    cells = np.zeros((len(frames), n), CELL)
    motion = np.zeros(len(frames), STILL_MOTION)
    hashes = np.zeros(len(frames), np.uint64)
    mean = np.zeros((h, w), np.float32)
    got = ref().ref_still_run(_p(buf), len(frames), stride, w, h, avg, C.c_float(motion_px), C.c_float(motion_grey),
                              _p(cells), _p(motion), _p(hashes), _p(mean))
    assert got == n
    return cells, motion, hashes, mean


# ---------------------------------------------------------------- frame generation (src/kern/framegen.c)

FG_VEC = np.dtype([("x", "<i2"), ("y", "<i2")])  # struct fg_vec


def fg_shapes(w: int, h: int):
    """The field's levels for w x h frames: [(level w, level h, blocks across, blocks down)], level 0 first."""
    out, lw, lh = [], (w + 1) // 2, (h + 1) // 2
    while len(out) < 7 and lw >= 16 and lh >= 16:
        out.append((lw, lh, (lw + 7) // 8, (lh + 7) // 8))
        lw, lh = (lw + 1) // 2, (lh + 1) // 2
    return out


def _fg_outputs(w, h):
    shapes = fg_shapes(w, h)
    total = sum(bw * bh for _, _, bw, bh in shapes)
    return (shapes, np.zeros(total, FG_VEC), np.zeros(total, FG_VEC), np.zeros(total, FG_VEC),
            np.zeros(shapes[0][2] * shapes[0][3], FG_VEC), np.zeros((h, w), np.float32), np.zeros((h, w), np.uint8))


def _fg_split(shapes, raw, fil, up, mid, out, pic, scene):
    res = {"scene": int(scene), "raw": [], "fil": [], "up": [], "mid": mid.reshape(shapes[0][3], shapes[0][2]),
           "out": out, "pic": pic}
    o = 0
    for _, _, bw, bh in shapes:
        for k, a in (("raw", raw), ("fil", fil), ("up", up)):
            res[k].append(a[o:o + bw * bh].reshape(bh, bw))
        o += bw * bh
    return res


def framegen(a0, b0):
    """The oracle's generated frame between Q6 planes a0 (older) and b0 (newer): a dict of the fields per level (raw,
    fil, up), mid, the frame (Q6) and its bytes, and the scene verdict."""
    a0 = np.ascontiguousarray(a0, np.float32)
    b0 = np.ascontiguousarray(b0, np.float32)
    h, w = a0.shape
    shapes, raw, fil, up, mid, out, pic = _fg_outputs(w, h)
    scene = lib().or_framegen(_p(a0), _p(b0), w, h, w, _p(raw), _p(fil), _p(up), _p(mid), _p(out), _p(pic))
    assert scene >= 0
    return _fg_split(shapes, raw, fil, up, mid, out, pic, scene)


def ref_framegen(fa, fb):
    """The reference's framegen.c on two 8-bit frames, the same dict."""
    h, w = fa.shape
    stride = (w + 15) & ~15
    ba = np.zeros((h, stride), np.uint8)
    bb = np.zeros((h, stride), np.uint8)
    ba[:, :w] = fa
    bb[:, :w] = fb
    shapes, raw, fil, up, mid, out, pic = _fg_outputs(w, h)
    scene = ref().ref_framegen(_p(ba), _p(bb), stride, w, h, _p(raw), _p(fil), _p(up), _p(mid), _p(out), _p(pic))
    assert scene >= 0
    return _fg_split(shapes, raw, fil, up, mid, out, pic, scene)
