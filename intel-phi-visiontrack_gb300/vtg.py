"""vtg.py -- Python binding of libvtg's C ABI (include/vtg.h), for tests, the benchmark and Python callers.

Loads the in-tree libvtg.so built by vtg_build.py and fails loudly when it is missing: there is no CPU or PyTorch
fallback behind any function here. numpy arrays in and out for host buffers; device buffers are raw addresses (for
example ``torch.Tensor.data_ptr()``) passed with ``where=DEVICE``.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# VTG_LIB names another build of the library (the bounds-checked libvtg_checked.so) for this process
LIB_PATH = os.environ.get("VTG_LIB") or os.path.join(HERE, "libvtg.so")

OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, EBUSY, ENODEV, EBUDGET = 0, -1, -2, -3, -4, -5, -6, -7
HOST, DEVICE = 0, 1
# tk_build's optional input steps (vtg_tracker_set_build): the contrast stretch and the 5 x 5 binomial
BUILD_CONTRAST, BUILD_PRE_GAUSS = 1, 2
LK_OK, LK_OUT, LK_LOWEIG, LK_RESIDUAL, LK_FLOWBACK = 0, 1, 2, 4, 8
MAX_LEVELS = 6

LK_OUT_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("min_eig", "<f4"), ("residual", "<f4"), ("cov_xx", "<f4"),
                         ("cov_xy", "<f4"), ("cov_yy", "<f4"), ("iters", "<u2"), ("status", "<u2")])
CELL_DTYPE = np.dtype([("u", "<f4"), ("v", "<f4"), ("diff", "<f4"), ("state", "<u4"), ("sigma", "<f4"),
                       ("pad", "<f4")])


class Config(C.Structure):
    """struct vtg_config."""
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("levels", C.c_uint32), ("patch_w", C.c_uint32),
                ("patch_h", C.c_uint32), ("max_iter", C.c_uint32), ("eps", C.c_float), ("min_eig", C.c_float),
                ("max_residual", C.c_float), ("fb_max", C.c_float), ("cell_w", C.c_uint32), ("cell_h", C.c_uint32),
                ("flow_level", C.c_uint32)]


def config(width, height, levels=4, patch_w=21, patch_h=21, max_iter=10, eps=0.01, min_eig=0.1, max_residual=25.0,
           fb_max=0.5, cell_w=16, cell_h=8, flow_level=0) -> Config:
    return Config(width, height, levels, patch_w, patch_h, max_iter, eps, min_eig, max_residual, fb_max, cell_w,
                  cell_h, flow_level)


class VtgError(RuntimeError):
    def __init__(self, code: int, what: str):
        msg = lib().vtg_strerror(code).decode()
        if code == ECUDA:
            msg += " (cudaError %d)" % lib().vtg_last_cuda_error()
        super().__init__("%s: %s" % (what, msg))
        self.code = code


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libvtg.so is not built (run vtg_build.py / __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        vp, sz, i, f = C.c_void_p, C.c_size_t, C.c_int, C.c_float
        L.vtg_strerror.restype = C.c_char_p
        L.vtg_strerror.argtypes = [i]
        L.vtg_last_cuda_error.restype = i
        L.vtg_ctx_create.argtypes = [i, sz, C.POINTER(vp)]
        L.vtg_ctx_destroy.argtypes = [vp]
        L.vtg_ctx_destroy.restype = None
        L.vtg_ctx_used.argtypes = [vp]
        L.vtg_ctx_used.restype = sz
        L.vtg_ctx_sync.argtypes = [vp, i]
        L.vtg_tracker_bytes.argtypes = [C.POINTER(Config)]
        L.vtg_tracker_bytes.restype = sz
        L.vtg_tracker_create.argtypes = [vp, C.POINTER(Config), C.POINTER(vp)]
        L.vtg_tracker_destroy.argtypes = [vp]
        L.vtg_tracker_destroy.restype = None
        L.vtg_tracker_sets.argtypes = [vp]
        L.vtg_tracker_cells.argtypes = [vp, C.POINTER(i), C.POINTER(i)]
        L.vtg_tracker_stream.argtypes = [vp]
        L.vtg_tracker_stream.restype = vp
        L.vtg_build.argtypes = [vp, i, vp, i, i, vp]
        L.vtg_cells.argtypes = [vp, i, i, vp, vp, i, vp]
        L.vtg_points.argtypes = [vp, i, i, i, i, vp, vp, vp, vp, vp, i, vp]
        L.vtg_level.argtypes = [vp, i, i, vp, i, vp]
        L.vtg_level_size.argtypes = [vp, i, C.POINTER(i), C.POINTER(i)]
        L.vtg_tracker_set_build.argtypes = [vp, i]
        L.vtg_tracker_set_point_warps.argtypes = [vp, i]
        L.vtg_tracker_build_flags.argtypes = [vp]
        L.vtg_contrast_gain.argtypes = [i, i, vp]
        L.vtg_store_appearance.argtypes = [vp, i, f, f, f, f, vp, vp, C.POINTER(Appearance), i, vp]
        L.vtg_check_read.argtypes = [vp]
        _lib = L
    return _lib


APP_W, APP_H = 32, 21


class Appearance(C.Structure):
    """struct vtg_appearance: where store_appearance cut its template."""
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("level", C.c_int32), ("valid", C.c_int32)]


def contrast_gain(lo: int, hi: int):
    """tk_build's stretch (gain, offset) as float32 for Q6 minimum lo and maximum hi (vtg_contrast_gain)."""
    go = np.zeros(2, np.float32)
    check(lib().vtg_contrast_gain(int(lo), int(hi), go.ctypes.data), "vtg_contrast_gain")
    return go


def check(code: int, what: str) -> int:
    if code < 0:
        raise VtgError(code, what)
    return code


def _p(a):
    return None if a is None else a.ctypes.data


class Context:
    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.h = C.c_void_p()
        self._trackers = weakref.WeakSet()
        check(lib().vtg_ctx_create(device, hbm_budget, C.byref(self.h)), "vtg_ctx_create")

    def used(self) -> int:
        return lib().vtg_ctx_used(self.h)

    def sync(self, timeout_ms: int = 10000):
        check(lib().vtg_ctx_sync(self.h, timeout_ms), "vtg_ctx_sync")

    def close(self):
        if self.h:
            for t in list(self._trackers):
                if isinstance(t, Tracker):
                    t.h = C.c_void_p()  # the context frees its trackers
                else:
                    t.close()
            lib().vtg_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tracker:
    """One stream's device-resident pyramids and cell results (vtg_tracker)."""

    def __init__(self, ctx: Context, cfg: Config):
        self.ctx = ctx
        self.cfg = cfg
        self.h = C.c_void_p()
        check(lib().vtg_tracker_create(ctx.h, C.byref(cfg), C.byref(self.h)), "vtg_tracker_create")
        ctx._trackers.add(self)
        cols, rows = C.c_int(), C.c_int()
        lib().vtg_tracker_cells(self.h, C.byref(cols), C.byref(rows))
        self.cols, self.rows = cols.value, rows.value

    @property
    def stream(self) -> int:
        return lib().vtg_tracker_stream(self.h)

    def sync(self, timeout_ms: int = 10000):
        self.ctx.sync(timeout_ms)

    def level_size(self, level: int):
        w, h = C.c_int(), C.c_int()
        check(lib().vtg_level_size(self.h, level, C.byref(w), C.byref(h)), "vtg_level_size")
        return w.value, h.value

    def build(self, set_: int, frame, stride: int | None = None, where: int = HOST, stream=None):
        if where == HOST:
            frame = np.ascontiguousarray(frame, np.uint8)
            stride = frame.shape[1] if stride is None else stride
            ptr = frame.ctypes.data
        else:
            ptr = frame
            stride = self.cfg.width if stride is None else stride
        check(lib().vtg_build(self.h, set_, ptr, stride, where, stream), "vtg_build")

    def store_appearance(self, set_: int, cx: float, cy: float, rw: float, rh: float) -> dict:
        """store_appearance from a set's resident pyramid: pix (21 x 32), norm, fx, fy, level, valid (host copies)."""
        a = Appearance()
        pix = np.zeros((APP_H, APP_W), np.float32)
        norm = np.zeros(1, np.float32)
        check(lib().vtg_store_appearance(self.h, set_, cx, cy, rw, rh, pix.ctypes.data, norm.ctypes.data,
                                         C.byref(a), HOST, None), "vtg_store_appearance")
        self.sync()
        return {"pix": pix, "norm": norm[0], "fx": np.float32(a.fx), "fy": np.float32(a.fy), "level": a.level,
                "valid": bool(a.valid)}

    def set_build(self, flags: int):
        """tk_build's optional steps for later builds: BUILD_CONTRAST | BUILD_PRE_GAUSS (0: neither)."""
        check(lib().vtg_tracker_set_build(self.h, int(flags)), "vtg_tracker_set_build")

    @property
    def build_flags(self) -> int:
        return lib().vtg_tracker_build_flags(self.h)

    def set_point_warps(self, warps: int):
        """Warps a point for later points() calls: 1, 2 (half the patch's rows each), or 0 (the default: 1)."""
        check(lib().vtg_tracker_set_point_warps(self.h, int(warps)), "vtg_tracker_set_point_warps")

    def level(self, set_: int, level: int) -> np.ndarray:
        w, h = self.level_size(level)
        out = np.empty((h, w), np.float32)
        check(lib().vtg_level(self.h, set_, level, _p(out), HOST, None), "vtg_level")
        self.sync()
        return out

    def cells(self, prev: int, cur: int, want_lk: bool = True):
        n = self.cols * self.rows
        cells = np.zeros(n, CELL_DTYPE)
        lk = np.zeros(n, LK_OUT_DTYPE) if want_lk else None
        check(lib().vtg_cells(self.h, prev, cur, _p(cells), _p(lk), HOST, None), "vtg_cells")
        self.sync()
        return cells, lk

    def cells_device(self, prev: int, cur: int, cells_ptr, lk_ptr, stream=None):
        check(lib().vtg_cells(self.h, prev, cur, cells_ptr, lk_ptr, DEVICE, stream), "vtg_cells")

    def points(self, prev: int, cur: int, xs, ys, gx=None, gy=None, top: int = -1) -> np.ndarray:
        xs = np.ascontiguousarray(xs, np.float32)
        ys = np.ascontiguousarray(ys, np.float32)
        gx = None if gx is None else np.ascontiguousarray(gx, np.float32)
        gy = None if gy is None else np.ascontiguousarray(gy, np.float32)
        out = np.zeros(len(xs), LK_OUT_DTYPE)
        check(lib().vtg_points(self.h, prev, cur, top, len(xs), _p(xs), _p(ys), _p(gx), _p(gy), _p(out), HOST, None),
              "vtg_points")
        self.sync()
        return out

    def close(self):
        if self.h:
            lib().vtg_tracker_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- the appearance search

PLANE_U8, PLANE_F32 = 0, 1
NCC_F32, NCC_BF16, NCC_FP16 = 0, 1, 2


class Found(C.Structure):
    """struct vtg_found."""
    _fields_ = [("hx", C.c_int), ("hy", C.c_int), ("ncc", C.c_float), ("second", C.c_float), ("ox", C.c_float),
                ("oy", C.c_float), ("ntop", C.c_int), ("cells", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def _search_sigs(L):
    vp, i, f, sz = C.c_void_p, C.c_int, C.c_float, C.c_size_t
    L.vtg_search_bytes.argtypes = [i, i, i, i]
    L.vtg_search_bytes.restype = sz
    L.vtg_search_create.argtypes = [vp, i, i, i, i, C.POINTER(vp)]
    L.vtg_search_destroy.argtypes = [vp]
    L.vtg_search_destroy.restype = None
    L.vtg_search_stream.argtypes = [vp]
    L.vtg_search_stream.restype = vp
    L.vtg_search_template.argtypes = [vp, vp, i, i, f, i, vp]
    L.vtg_search_run.argtypes = [vp, vp, i, i, i, i, i, i, i, i, i, i, C.POINTER(Found), vp, vp, vp, i, vp]
    L.vtg_correlate.argtypes = [vp, vp, i, i, i, i, i, vp, vp, vp, i, vp]
    L.vtg_search_profile.argtypes = [vp, vp, i, i, i, i, i, i, i, i, i, i, i, C.POINTER(f), C.POINTER(f)]
    L.vtg_level_device.argtypes = [vp, i, i, C.POINTER(vp), C.POINTER(i), C.POINTER(i), C.POINTER(i)]


class Search:
    """A search context (vtg_search): a template and the scratch of its searches."""

    def __init__(self, ctx: Context, max_w: int, max_h: int, max_tw: int = 128, max_th: int = 128):
        _search_sigs(lib())
        self.ctx = ctx
        self.h = C.c_void_p()
        check(lib().vtg_search_create(ctx.h, max_w, max_h, max_tw, max_th, C.byref(self.h)), "vtg_search_create")
        ctx._trackers.add(self)

    def template(self, app, norm: float):
        app = np.ascontiguousarray(app, np.float32)
        check(lib().vtg_search_template(self.h, _p(app), app.shape[1], app.shape[0], C.c_float(norm), HOST, None),
              "vtg_search_template")

    def run(self, plane_ptr: int, w: int, h: int, pitch: int, plane_type: int, x0: int, x1: int, y0: int, y1: int,
            step: int = 1, precision: int = NCC_F32, want_map: bool = False):
        f = Found()
        ncell = (w // 16 + 2) * (h // 16 + 2)
        mv = np.zeros(ncell, np.float32) if want_map else None
        mx = np.zeros(ncell, np.int32) if want_map else None
        my = np.zeros(ncell, np.int32) if want_map else None
        check(lib().vtg_search_run(self.h, plane_ptr, w, h, pitch, plane_type, x0, x1, y0, y1, step, precision,
                                   C.byref(f), _p(mv), _p(mx), _p(my), HOST, None), "vtg_search_run")
        d = f.as_dict()
        if want_map:
            n = d["cells"]
            return d, mv[:n], mx[:n], my[:n]
        return d

    def profile(self, plane_ptr: int, w: int, h: int, pitch: int, plane_type: int, x0: int, x1: int, y0: int, y1: int,
                step: int = 1, precision: int = NCC_F32, reps: int = 10):
        """(map kernel ms, whole search ms): medians of reps CUDA-event timed runs (vtg_search_profile)."""
        a, b = C.c_float(), C.c_float()
        check(lib().vtg_search_profile(self.h, plane_ptr, w, h, pitch, plane_type, x0, x1, y0, y1, step, precision,
                                       reps, C.byref(a), C.byref(b)), "vtg_search_profile")
        return a.value, b.value

    def correlate(self, plane_ptr: int, w: int, h: int, pitch: int, plane_type: int, xs, ys) -> np.ndarray:
        xs = np.ascontiguousarray(xs, np.int32)
        ys = np.ascontiguousarray(ys, np.int32)
        out = np.zeros(len(xs), np.float32)
        check(lib().vtg_correlate(self.h, plane_ptr, w, h, pitch, plane_type, len(xs), _p(xs), _p(ys), _p(out), HOST,
                                  None), "vtg_correlate")
        return out

    def close(self):
        if self.h:
            lib().vtg_search_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def level_device(tracker: Tracker, set_: int, level: int):
    """(device address, w, h, pitch) of a tracker's pyramid level (F32 Q6)."""
    _search_sigs(lib())
    p, w, h, pitch = C.c_void_p(), C.c_int(), C.c_int(), C.c_int()
    check(lib().vtg_level_device(tracker.h, set_, level, C.byref(p), C.byref(w), C.byref(h), C.byref(pitch)),
          "vtg_level_device")
    return p.value, w.value, h.value, pitch.value


# ---------------------------------------------------------------- many streams in one step

class Tune(C.Structure):
    """struct vtg_tune."""
    _fields_ = [("block_warps", C.c_int), ("chunk", C.c_int), ("persistent", C.c_int), ("ctas_per_sm", C.c_int),
                ("tsmem", C.c_int), ("tiled", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def _batch_sigs(L):
    vp, i = C.c_void_p, C.c_int
    L.vtg_batch_create.argtypes = [vp, i, C.POINTER(vp)]
    L.vtg_batch_destroy.argtypes = [vp]
    L.vtg_batch_destroy.restype = None
    L.vtg_batch_stream.argtypes = [vp]
    L.vtg_batch_stream.restype = vp
    L.vtg_batch_prepare.argtypes = [vp, i, i, C.POINTER(vp), C.POINTER(vp), C.POINTER(i), i, C.POINTER(i)]
    L.vtg_batch_launch.argtypes = [vp, i, vp]
    L.vtg_batch_capture.argtypes = [vp, i]
    L.vtg_batch_replay.argtypes = [vp, i, vp]
    L.vtg_batch_cells.argtypes = [vp, i]
    L.vtg_batch_set_tune.argtypes = [vp, C.POINTER(Tune)]
    L.vtg_batch_get_tune.argtypes = [vp, C.POINTER(Tune)]
    L.vtg_batch_autotune.argtypes = [vp, i, i, C.POINTER(Tune), C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.vtg_tracker_results.argtypes = [vp, vp, vp, i, vp]
    L.vtg_batch_profile.argtypes = [vp, i, i, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.vtg_batch_count.argtypes = [vp, i, C.POINTER(C.c_uint64)]


class Batch:
    """A batch (vtg_batch): many trackers' frame pairs in one step, graph-capturable, autotuned."""

    def __init__(self, ctx: Context, max_jobs: int):
        _batch_sigs(lib())
        self.ctx = ctx
        self.h = C.c_void_p()
        check(lib().vtg_batch_create(ctx.h, max_jobs, C.byref(self.h)), "vtg_batch_create")
        ctx._trackers.add(self)
        self._keep = {}

    @property
    def stream(self) -> int:
        return lib().vtg_batch_stream(self.h)

    def prepare(self, slot: int, trackers, frames, cur_sets, where: int = DEVICE, strides=None):
        """frames: device addresses (where=DEVICE) or uint8 numpy arrays (where=HOST; kept alive here)."""
        n = len(trackers)
        th = (C.c_void_p * n)(*[t.h.value for t in trackers])
        if where == HOST:
            arrs = [np.ascontiguousarray(f, np.uint8) for f in frames]
            self._keep[slot] = arrs
            ptrs = [a.ctypes.data for a in arrs]
            strides = strides or [a.shape[1] for a in arrs]
        else:
            ptrs = list(frames)
        fp = (C.c_void_p * n)(*ptrs)
        sp = (C.c_int * n)(*strides) if strides is not None else None
        cs = (C.c_int * n)(*cur_sets)
        check(lib().vtg_batch_prepare(self.h, slot, n, th, fp, sp, where, cs), "vtg_batch_prepare")

    def launch(self, slot: int, stream=None):
        check(lib().vtg_batch_launch(self.h, slot, stream), "vtg_batch_launch")

    def capture(self, slot: int):
        check(lib().vtg_batch_capture(self.h, slot), "vtg_batch_capture")

    def replay(self, slot: int, stream=None):
        check(lib().vtg_batch_replay(self.h, slot, stream), "vtg_batch_replay")

    def cells(self, slot: int) -> int:
        return check(lib().vtg_batch_cells(self.h, slot), "vtg_batch_cells")

    def set_tune(self, **kw):
        t = Tune()
        check(lib().vtg_batch_get_tune(self.h, C.byref(t)), "vtg_batch_get_tune")
        for k, v in kw.items():
            setattr(t, k, v)
        check(lib().vtg_batch_set_tune(self.h, C.byref(t)), "vtg_batch_set_tune")

    def get_tune(self) -> dict:
        t = Tune()
        check(lib().vtg_batch_get_tune(self.h, C.byref(t)), "vtg_batch_get_tune")
        return t.as_dict()

    def autotune(self, slot: int, reps: int = 5):
        t = Tune()
        b, d = C.c_float(), C.c_float()
        check(lib().vtg_batch_autotune(self.h, slot, reps, C.byref(t), C.byref(b), C.byref(d)), "vtg_batch_autotune")
        return t.as_dict(), b.value, d.value

    def profile(self, slot: int, reps: int = 5):
        """(pyramid ms, LK ms): medians over reps runs of the prepared step."""
        a, b = C.c_float(), C.c_float()
        check(lib().vtg_batch_profile(self.h, slot, reps, C.byref(a), C.byref(b)), "vtg_batch_profile")
        return a.value, b.value

    def count(self, slot: int) -> dict:
        """The work of one LK launch of the prepared step, both walks of every cell: template builds, residual passes,
        window passes, iterations (vtg_batch_count)."""
        c = (C.c_uint64 * 4)()
        check(lib().vtg_batch_count(self.h, slot, c), "vtg_batch_count")
        return {"builds": int(c[0]), "residuals": int(c[1]), "passes": int(c[2]), "iterations": int(c[3])}

    def close(self):
        if self.h:
            lib().vtg_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tracker_results(t: Tracker, want_lk: bool = True):
    _batch_sigs(lib())
    n = t.cols * t.rows
    cells = np.zeros(n, CELL_DTYPE)
    lk = np.zeros(n, LK_OUT_DTYPE) if want_lk else None
    check(lib().vtg_tracker_results(t.h, _p(cells), _p(lk), HOST, None), "vtg_tracker_results")
    t.ctx.sync()
    return cells, lk


# ---------------------------------------------------------------- the served request loop

class ServeStream(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("flow_level", C.c_uint32), ("fps", C.c_float),
                ("start_s", C.c_float), ("frames", C.c_int)]


class ServeCfg(C.Structure):
    _fields_ = [("nstreams", C.c_int), ("streams", C.POINTER(ServeStream)), ("frames", C.POINTER(C.c_void_p)),
                ("lk", Config), ("duration_s", C.c_double), ("max_batch", C.c_int), ("inflight", C.c_int),
                ("hbm_budget", C.c_size_t), ("ncc_share", C.c_float), ("plain", C.c_int), ("seed", C.c_uint64),
                ("last_cells", C.POINTER(C.c_void_p)), ("live", C.c_int), ("max_queue", C.c_int),
                ("stall_at_s", C.c_double), ("stall_timeout_s", C.c_double)]


class ServeStats(C.Structure):
    _fields_ = [("streams_admitted", C.c_int), ("streams_waited", C.c_int), ("streams_rejected", C.c_int),
                ("requests", C.c_long), ("served", C.c_long), ("cells", C.c_long), ("ncc", C.c_long),
                ("wall_s", C.c_double), ("cells_per_s", C.c_double), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("max_ms", C.c_double), ("mean_batch", C.c_double), ("skipped", C.c_long), ("dropped", C.c_long),
                ("submitted", C.c_long)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def serve(ctx: Context, streams, frames, lk: Config, duration_s: float, max_batch: int = 64, inflight: int = 2,
          hbm_budget: int = 0, ncc_share: float = 0.0, plain: bool = False, seed: int = 1, last_cells=None,
          live: bool = False, max_queue: int = 0, stall_at_s: float = 0.0, stall_timeout_s: float = 0.0,
          allow_timeout: bool = False) -> dict:
    """Runs vtg_serve_run. streams: dicts (width, height, flow_level, fps, start_s, frames); frames: two host
    addresses per stream (pinned uint8 buffers, width bytes a row); last_cells: optional list of CELL_DTYPE arrays
    (cols x rows each, or None) that end with each stream's last frame pair's cells. With allow_timeout, a
    VTG_ETIMEOUT run returns its stats with "rc" set instead of raising."""
    L = lib()
    L.vtg_serve_run.argtypes = [C.c_void_p, C.POINTER(ServeCfg), C.POINTER(ServeStats)]
    ss = (ServeStream * len(streams))(*[ServeStream(s["width"], s["height"], s.get("flow_level", 0), s["fps"],
                                                     s.get("start_s", 0.0), s["frames"]) for s in streams])
    fp = (C.c_void_p * len(frames))(*frames)
    lc = None
    if last_cells is not None:
        lc = (C.c_void_p * len(streams))(*[None if a is None else a.ctypes.data for a in last_cells])
    cfg = ServeCfg(len(streams), ss, fp, lk, duration_s, max_batch, inflight, hbm_budget, ncc_share, int(plain), seed,
                   lc, int(live), max_queue, stall_at_s, stall_timeout_s)
    st = ServeStats()
    rc = L.vtg_serve_run(ctx.h, C.byref(cfg), C.byref(st))
    if not (allow_timeout and rc == ETIMEOUT):
        check(rc, "vtg_serve_run")
    d = st.as_dict()
    d["rc"] = rc
    return d


# ---------------------------------------------------------------- the request API (vtg_server_*)

PRIO_ORDERED, PRIO_LIVE = 0, 1
REQ_SEARCH = 1
RES_DONE, RES_SKIPPED, RES_RETIRED = 0, 1, 2


class ServerCfg(C.Structure):
    _fields_ = [("lk", Config), ("max_batch", C.c_int), ("inflight", C.c_int), ("plain", C.c_int),
                ("max_queue", C.c_int), ("idle_timeout_s", C.c_double)]


class ServerResult(C.Structure):
    _fields_ = [("stream", C.c_int), ("status", C.c_int), ("ticket", C.c_int64), ("tag", C.c_uint64),
                ("frames_skipped", C.c_uint32), ("searched", C.c_int), ("latency_ms", C.c_double), ("found", Found)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "found"}
        d["found"] = self.found.as_dict()
        return d


def _server_sigs(L):
    vp, i, i64 = C.c_void_p, C.c_int, C.c_int64
    L.vtg_server_create.argtypes = [vp, C.POINTER(ServerCfg), C.POINTER(vp)]
    L.vtg_server_destroy.argtypes = [vp]
    L.vtg_server_destroy.restype = None
    L.vtg_server_template.argtypes = [vp, vp, i, i, C.c_float]
    L.vtg_server_open.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, i, vp, i]
    L.vtg_server_close.argtypes = [vp, i]
    L.vtg_server_submit.argtypes = [vp, i, vp, i, vp, C.c_uint64, i]
    L.vtg_server_submit.restype = i64
    L.vtg_server_poll.argtypes = [vp, C.POINTER(ServerResult), i, i]
    L.vtg_server_pending.argtypes = [vp]
    L.vtg_server_counts.argtypes = [vp, C.POINTER(C.c_long), C.POINTER(C.c_long)]


class Server:
    """The request API (vtg_server): open streams, submit frames as they arrive, poll for their cells."""

    def __init__(self, ctx: Context, lk: Config, max_batch: int = 64, inflight: int = 2, plain: bool = False,
                 max_queue: int = 16, idle_timeout_s: float = 0.0):
        _server_sigs(lib())
        self.ctx = ctx
        self.h = C.c_void_p()
        cfg = ServerCfg(lk, max_batch, inflight, int(plain), max_queue, idle_timeout_s)
        check(lib().vtg_server_create(ctx.h, C.byref(cfg), C.byref(self.h)), "vtg_server_create")
        ctx._trackers.add(self)
        self._keep = {}
        self._widths = {}

    def template(self, app, norm: float):
        app = np.ascontiguousarray(app, np.float32)
        check(lib().vtg_server_template(self.h, _p(app), app.shape[1], app.shape[0], C.c_float(norm)),
              "vtg_server_template")

    def open(self, width: int, height: int, first, flow_level: int = 0, priority: int = PRIO_ORDERED,
             stride: int = 0) -> int:
        """A stream id (>= 0) or a negative status (not raised: EINVAL and EBUDGET are answers here)."""
        sid = lib().vtg_server_open(self.h, width, height, flow_level, priority, first, stride or width)
        if sid >= 0:
            self._widths[sid] = width
        return sid

    def close_stream(self, stream: int) -> int:
        return lib().vtg_server_close(self.h, stream)

    def submit(self, stream: int, frame, cells=None, tag: int = 0, flags: int = 0, stride: int = 0) -> int:
        """frame: a host address (pinned); cells: a CELL_DTYPE array (kept alive until polled) or None."""
        t = lib().vtg_server_submit(self.h, stream, frame, stride or self._width(stream), _p(cells), tag, flags)
        if t >= 0 and cells is not None:
            self._keep[t] = cells
        return t

    def _width(self, stream: int) -> int:
        return self._widths.get(stream, 0)

    def poll(self, max_results: int = 256, timeout_us: int = 0):
        out = (ServerResult * max_results)()
        n = check(lib().vtg_server_poll(self.h, out, max_results, timeout_us), "vtg_server_poll")
        res = [out[i].as_dict() for i in range(n)]
        for r in res:
            self._keep.pop(r["ticket"], None)
        return res

    def pending(self) -> int:
        return check(lib().vtg_server_pending(self.h), "vtg_server_pending")

    def counts(self):
        a, b = C.c_long(), C.c_long()
        check(lib().vtg_server_counts(self.h, C.byref(a), C.byref(b)), "vtg_server_counts")
        return a.value, b.value

    def close(self):
        if self.h:
            lib().vtg_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- the reference's kernel signatures (vtg_compat.h)

class RefPlane(C.Structure):
    """struct vtg_ref_plane: the reference's struct vt_plane (pixel (0, 0), w, h, stride in floats)."""
    _fields_ = [("p", C.c_void_p), ("w", C.c_int), ("h", C.c_int), ("stride", C.c_int)]


class RefLkCfg(C.Structure):
    """struct vtg_ref_lk_cfg: the reference's struct lk_cfg."""
    _fields_ = [("w", C.c_int), ("h", C.c_int), ("max_iter", C.c_int), ("eps", C.c_float), ("min_eig", C.c_float),
                ("max_residual", C.c_float), ("prefetch", C.c_int)]


def compat() -> C.CDLL:
    """The library with the vtg_compat.h signatures set."""
    L = lib()
    if not getattr(L, "_compat_sigs", False):
        P, PL, i, f, vp = C.POINTER(RefPlane), C.POINTER(RefPlane), C.c_int, C.c_float, C.c_void_p
        L.lk_tile_bytes_cuda.restype = C.c_size_t
        L.img_u8_to_q6_cuda.argtypes = [P, vp, i, i, i]
        L.img_u8_to_q6_cuda.restype = None
        L.img_reduce_cuda.argtypes = [P, P, i, i]
        L.img_reduce_cuda.restype = None
        L.img_norm_cuda.argtypes = [P, P, vp, i, i]
        L.img_norm_cuda.restype = None
        L.img_minmax_cuda.argtypes = [P, vp, i, i]
        L.img_minmax_cuda.restype = None
        L.img_gauss5_cuda.argtypes = [P, P, i, i]
        L.img_gauss5_cuda.restype = None
        L.img_sobel_cuda.argtypes = [P, P, P, i, i]
        L.img_sobel_cuda.restype = None
        L.img_absdiff_cuda.argtypes = [P, P, P, i, i]
        L.img_absdiff_cuda.restype = None
        L.lk_track_cuda.argtypes = [PL, PL, i, C.POINTER(RefLkCfg), f, f, f, f, vp, vp]
        L.lk_track_cuda.restype = None
        L.lk_flowback_cuda.argtypes = [PL, PL, i, C.POINTER(RefLkCfg), f, f, f, vp, vp]
        L.lk_flowback_cuda.restype = None
        L.still_vectors_cuda.argtypes = [P, P, C.POINTER(RefLkCfg), f, vp, i, i]
        L.still_vectors_cuda.restype = None
        L.tk_correlate_cuda.argtypes = [P, vp, C.c_longdouble, i, i]
        L.tk_correlate_cuda.restype = C.c_longdouble
        L.detect_run_cuda.argtypes = [P, f, f, f, f, i, i, f, f, vp, vp]
        L.detect_run_cuda.restype = i
        L.vtg_compat_error.restype = C.c_int
        L._compat_sigs = True
    return L


# ---------------------------------------------------------------- corner detection

class Detector:
    """A corner detector (vtg_detector): detect_begin .. detect_finish of the reference on the GPU."""

    def __init__(self, ctx: Context, max_w: int, max_h: int):
        L = lib()
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        L.vtg_detector_create.argtypes = [vp, i, i, C.POINTER(vp)]
        L.vtg_detector_destroy.argtypes = [vp]
        L.vtg_detector_destroy.restype = None
        L.vtg_detector_stream.argtypes = [vp]
        L.vtg_detector_stream.restype = vp
        L.vtg_detect.argtypes = [vp, vp, i, i, i, f, f, f, f, i, i, f, f, vp, vp, vp, i, vp]
        L.vtg_detect_maps.argtypes = [vp, f, f, f, f, i, i, i, vp, vp, vp]
        self.ctx = ctx
        self.h = C.c_void_p()
        check(L.vtg_detector_create(ctx.h, max_w, max_h, C.byref(self.h)), "vtg_detector_create")
        ctx._trackers.add(self)

    def detect(self, plane_ptr: int, w: int, h: int, pitch: int, rx, ry, rw, rh, margin: int, max_n: int,
               min_dist: float, quality: float):
        """(xs, ys), best first: the corners of a device Q6 plane."""
        xs = np.zeros(max(max_n, 1), np.float32)
        ys = np.zeros(max(max_n, 1), np.float32)
        n = C.c_int()
        check(lib().vtg_detect(self.h, plane_ptr, w, h, pitch, rx, ry, rw, rh, margin, max_n, min_dist, quality,
                               _p(xs), _p(ys), C.byref(n), HOST, None), "vtg_detect")
        return xs[:n.value].copy(), ys[:n.value].copy()

    def maps(self, rx, ry, rw, rh, w: int, h: int, margin: int):
        """(geometry dict, resp, cells) of the last detect."""
        geo = np.zeros(9, np.int32)
        check(lib().vtg_detect_maps(self.h, rx, ry, rw, rh, w, h, margin, _p(geo), None, None), "vtg_detect_maps")
        g = dict(zip(("x0", "y0", "x1", "y1", "ax", "cols", "rows", "nv", "cell_rows"), [int(v) for v in geo]))
        resp = np.zeros((g["rows"], g["cols"]), np.float32)
        cell = np.zeros((g["cell_rows"], g["nv"]), np.float32)
        check(lib().vtg_detect_maps(self.h, rx, ry, rw, rh, w, h, margin, _p(geo), _p(resp), _p(cell)),
              "vtg_detect_maps")
        return g, resp, cell

    def close(self):
        if self.h:
            lib().vtg_detector_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


FG_VEC = np.dtype([("x", "<i2"), ("y", "<i2")])  # struct vtg_fg_vec


class Framegen:
    """Frame generation (vtg_framegen): the motion field between two frames and the frame between them."""

    def __init__(self, ctx: Context, w: int, h: int):
        L = lib()
        vp, i = C.c_void_p, C.c_int
        L.vtg_framegen_bytes.argtypes = [i, i]
        L.vtg_framegen_bytes.restype = C.c_size_t
        L.vtg_framegen_create.argtypes = [vp, i, i, C.POINTER(vp)]
        L.vtg_framegen_destroy.argtypes = [vp]
        L.vtg_framegen_destroy.restype = None
        L.vtg_framegen_stream.argtypes = [vp]
        L.vtg_framegen_stream.restype = vp
        L.vtg_framegen_levels.argtypes = [vp]
        L.vtg_framegen_run.argtypes = [vp, vp, i, vp, i, vp, i, vp, i, vp]
        L.vtg_framegen_fields.argtypes = [vp, i, vp, vp, vp, vp, vp, i, vp]
        L.vtg_framegen_frame.argtypes = [vp, C.POINTER(vp), C.POINTER(i)]
        self.ctx, self.w, self.h_ = ctx, w, h
        self.h = C.c_void_p()
        check(L.vtg_framegen_create(ctx.h, w, h, C.byref(self.h)), "vtg_framegen_create")
        ctx._trackers.add(self)
        self.levels = L.vtg_framegen_levels(self.h)
        self.shapes = []
        lw, lh = (w + 1) // 2, (h + 1) // 2
        for _ in range(self.levels):
            self.shapes.append((lw, lh, (lw + 7) // 8, (lh + 7) // 8))
            lw, lh = (lw + 1) // 2, (lh + 1) // 2

    def run(self, older_ptr: int, older_pitch: int, newer_ptr: int, newer_pitch: int, pic: bool = True):
        """One generated frame between two device Q6 planes: its bytes (h x w) when pic, else None."""
        out = np.zeros((self.h_, self.w), np.uint8) if pic else None
        check(lib().vtg_framegen_run(self.h, older_ptr, older_pitch, newer_ptr, newer_pitch, None, 0,
                                     None if out is None else _p(out), HOST, None), "vtg_framegen_run")
        return out

    def fields(self):
        """{raw, fil, up: per level (bh x bw FG_VEC), mid, scene} of the last run."""
        res = {"raw": [], "fil": [], "up": []}
        _, _, bw0, bh0 = self.shapes[0]
        mid = np.zeros((bh0, bw0), FG_VEC)
        scene = C.c_int()
        for L, (_, _, bw, bh) in enumerate(self.shapes):
            a = [np.zeros((bh, bw), FG_VEC) for _ in range(3)]
            check(lib().vtg_framegen_fields(self.h, L, _p(a[0]), _p(a[1]), _p(a[2]), _p(mid) if L == 0 else None,
                                            C.byref(scene) if L == 0 else None, HOST, None), "vtg_framegen_fields")
            for k, x in zip(("raw", "fil", "up"), a):
                res[k].append(x)
        res["mid"] = mid
        res["scene"] = scene.value
        return res

    def frame_ptr(self):
        """(device address, pitch in floats) of the last generated frame (Q6) inside the generator."""
        p, pitch = C.c_void_p(), C.c_int()
        check(lib().vtg_framegen_frame(self.h, C.byref(p), C.byref(pitch)), "vtg_framegen_frame")
        return p.value, pitch.value

    def stream(self):
        return lib().vtg_framegen_stream(self.h)

    def close(self):
        if self.h:
            lib().vtg_framegen_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StillConfig(C.Structure):
    """struct vtg_still_config: still_cfg (src/kern/still.h:21-27) without its thread count."""
    _fields_ = [("w", C.c_int), ("h", C.c_int), ("avg", C.c_int), ("motion_px", C.c_float),
                ("motion_grey", C.c_float)]


# struct vtg_still_motion: what still_motion fills (src/kern/still.c:262-275), 48 bytes.
STILL_MOTION = np.dtype([("cols", "<u4"), ("rows", "<u4"), ("tracked", "<u4"), ("moving", "<u4"),
                         ("count_mean", "<f4"), ("drift_u", "<f4"), ("drift_v", "<f4"), ("drift_rms", "<f4"),
                         ("diff_median", "<f4"), ("diff_limit", "<f4"), ("frames", "<u8")])


class Still:
    """One camera's still picture (vtg_still): still_vectors, still_decide, still_update, still_finish a frame."""

    def __init__(self, ctx: Context, w: int, h: int, avg: int = 8, motion_px: float = 1.0, motion_grey: float = 4.0):
        L = lib()
        vp, i = C.c_void_p, C.c_int
        L.vtg_still_bytes.argtypes = [C.POINTER(StillConfig)]
        L.vtg_still_bytes.restype = C.c_size_t
        L.vtg_still_create.argtypes = [vp, C.POINTER(StillConfig), C.POINTER(vp)]
        L.vtg_still_destroy.argtypes = [vp]
        L.vtg_still_destroy.restype = None
        L.vtg_still_stream.argtypes = [vp]
        L.vtg_still_stream.restype = vp
        L.vtg_still_frame.argtypes = [vp, vp, i, vp, i, vp]
        L.vtg_still_read.argtypes = [vp, vp, vp, vp, i, i, vp]
        L.vtg_still_mean.argtypes = [vp, C.POINTER(vp), C.POINTER(i)]
        self.ctx, self.w, self.h_ = ctx, w, h
        self.cols, self.rows = (w + 15) // 16, (h + 7) // 8
        self.cfg = StillConfig(w, h, avg, motion_px, motion_grey)
        self.h = C.c_void_p()
        check(L.vtg_still_create(ctx.h, C.byref(self.cfg), C.byref(self.h)), "vtg_still_create")
        ctx._trackers.add(self)

    def frame(self, cur_ptr: int, pitch: int, cells=None, stream=None):
        """One frame on a device Q6 plane; cells (a host CELL array) replaces the GPU's own vectors."""
        c = None if cells is None else np.ascontiguousarray(cells, CELL_DTYPE)
        check(lib().vtg_still_frame(self.h, cur_ptr, pitch, None if c is None else _p(c), HOST, stream),
              "vtg_still_frame")

    def read(self):
        """(cells, motion record, mean plane) of the newest frame."""
        cells = np.zeros(self.cols * self.rows, CELL_DTYPE)
        m = np.zeros(1, STILL_MOTION)
        mean = np.zeros((self.h_, self.w), np.float32)
        check(lib().vtg_still_read(self.h, _p(cells), _p(m), _p(mean), self.w, HOST, None), "vtg_still_read")
        return cells, m[0], mean

    def stream(self):
        return lib().vtg_still_stream(self.h)

    def close(self):
        if self.h:
            lib().vtg_still_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
