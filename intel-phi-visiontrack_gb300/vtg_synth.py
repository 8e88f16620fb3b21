"""vtg_synth.py -- seeded synthetic frames for the benchmark configurations of the LK path.

The reference measures on its own synthetic scenes and on private live frames; this generator stands in for both with
inputs of the same shapes and value ranges:

* ``noise_frame``: uniform 8-bit noise blurred by a Gaussian of sigma 1.5 px (11 integer taps summing to 2^16, applied
  separably with clamp-to-edge borders), kept as exact rationals, rounded and clipped to 0..255.
* ``warp_pair``: frame 1 is frame 0's continuous (pre-rounding) image, bilinearly resampled at x - d(x, y), so that the
  picture moves by +d: a global shift plus a smooth random field (a cubic B-spline through a seeded control grid)
  of amplitude at most ``amp`` px.
* ``ncc_templates``: T x T templates cut from a frame at seeded corners, then gain U(0.8, 1.2), offset U(-20, 20) and
  approximately Gaussian noise (sigma 3, the Irwin-Hall sum of 12 uniforms), rounded and clipped; a tenth of them are
  replaced by near-blank patches (standard deviation below 2).

Every random number comes from a counter-based splitmix64 hash in integer arithmetic, and every floating-point step is
an IEEE add, multiply or floor in numpy, so the bytes are the same on x86 and on Arm hosts and across numpy versions.
"""
from __future__ import annotations

import numpy as np

# exp(-k^2 / (2 * 1.5^2)) for k = -5..5, normalised and rounded to sum to 2^16.
GAUSS_TAPS = np.array([67, 498, 2359, 7167, 13960, 17434, 13960, 7167, 2359, 498, 67], np.int64)
assert int(GAUSS_TAPS.sum()) == 1 << 16

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def hash_u64(seed: int, stream: int, n: int) -> np.ndarray:
    """n 64-bit hashes of (seed, stream, 0..n-1)."""
    base = np.uint64(((((seed & 0xFFFFFFFF) << 32) ^ ((stream & 0xFFFF) << 16)) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF)
    idx = np.arange(n, dtype=np.uint64)
    return _splitmix(_splitmix(idx ^ base) ^ np.uint64(stream * 0x632BE59BD9B4E019 & 0xFFFFFFFFFFFFFFFF))


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n uniforms in [0, 1), 53 bits each."""
    return (hash_u64(seed, stream, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _blur_axis(a: np.ndarray, axis: int) -> np.ndarray:
    n = a.shape[axis]
    out = np.zeros(a.shape, np.int64)
    for k, t in enumerate(GAUSS_TAPS):
        idx = np.clip(np.arange(n) + (k - 5), 0, n - 1)
        out += int(t) * np.take(a, idx, axis=axis)
    return out


def blurred_noise(w: int, h: int, seed: int) -> np.ndarray:
    """The continuous image: uniform noise 0..255 blurred at sigma 1.5, float64 (an exact multiple of 2^-32)."""
    noise = (hash_u64(seed, 1, w * h) >> np.uint64(56)).astype(np.int64).reshape(h, w)
    s = _blur_axis(_blur_axis(noise, 1), 0)  # sum < 255 * 2^32: exact in int64
    return s.astype(np.float64) * (1.0 / 4294967296.0)


def to_u8(img: np.ndarray) -> np.ndarray:
    return np.clip(np.floor(img + 0.5), 0, 255).astype(np.uint8)


def noise_frame(w: int, h: int, seed: int) -> np.ndarray:
    return to_u8(blurred_noise(w, h, seed))


def _bspline_weights(t: np.ndarray):
    t2 = t * t
    t3 = t2 * t
    return ((1.0 - t) ** 3 / 6.0, (3.0 * t3 - 6.0 * t2 + 4.0) / 6.0, (-3.0 * t3 + 3.0 * t2 + 3.0 * t + 1.0) / 6.0,
            t3 / 6.0)


def smooth_field(w: int, h: int, seed: int, stream: int, grid=(8, 6)) -> np.ndarray:
    """A smooth field in [-1, 1]: a cubic B-spline through a (gx + 3) x (gy + 3) grid of seeded values, its largest
    magnitude scaled to 1."""
    gx, gy = grid
    ctrl = (uniform(seed, stream, (gx + 3) * (gy + 3)) * 2.0 - 1.0).reshape(gy + 3, gx + 3)
    ux = (np.arange(w, dtype=np.float64) + 0.5) * (gx / w)
    uy = (np.arange(h, dtype=np.float64) + 0.5) * (gy / h)
    ix, iy = np.floor(ux).astype(np.int64), np.floor(uy).astype(np.int64)
    wx, wy = _bspline_weights(ux - ix), _bspline_weights(uy - iy)
    # separable: rows of the control grid first, then columns
    rows = np.zeros((gy + 3, w))
    for k in range(4):
        rows += wx[k][None, :] * ctrl[:, ix + k]
    f = np.zeros((h, w))
    for k in range(4):
        f += wy[k][:, None] * rows[iy + k, :]
    m = np.max(np.abs(f))
    return f / m if m > 0 else f


def displacement(w: int, h: int, shift, amp: float, seed: int):
    """The displacement (dx, dy) per pixel of frame 1: the global shift plus fields of amplitude <= amp."""
    dx = shift[0] + amp * smooth_field(w, h, seed, 11)
    dy = shift[1] + amp * smooth_field(w, h, seed, 12)
    return dx, dy


def bilinear(img: np.ndarray, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    h, w = img.shape
    x = np.clip(x, 0.0, w - 1.0)
    y = np.clip(y, 0.0, h - 1.0)
    x0 = np.minimum(np.floor(x).astype(np.int64), w - 2)
    y0 = np.minimum(np.floor(y).astype(np.int64), h - 2)
    fx, fy = x - x0, y - y0
    a, b = img[y0, x0], img[y0, x0 + 1]
    c, d = img[y0 + 1, x0], img[y0 + 1, x0 + 1]
    top = a + fx * (b - a)
    bot = c + fx * (d - c)
    return top + fy * (bot - top)


def warp_pair(w: int, h: int, shift=(1.7, -0.8), amp: float = 0.5, seed: int = 1):
    """(frame 0, frame 1, dx, dy): frame 1 is frame 0 moved by (dx, dy) at each pixel of frame 1."""
    base = blurred_noise(w, h, seed)
    dx, dy = displacement(w, h, shift, amp, seed)
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float64)
    moved = bilinear(base, xs - dx, ys - dy)
    return to_u8(base), to_u8(moved), dx, dy


def still_sequence(w: int, h: int, frames: int, seed: int, jump_at: int | None = None, mover: int = 24):
    """A still camera's frames over a room: the blurred-noise scene drifting 0.03 px right and 0.02 px down a frame
    (the camera against its own past), sensor noise uniform in [-3, 3) grey each frame, a textured square of `mover`
    px entering at frame 2 and moving 3 px right a frame, and from frame `jump_at` on the whole picture 40 grey
    brighter (a light turned on: everything changed)."""
    base = blurred_noise(w, h, seed)
    tex = blurred_noise(mover, mover, seed + 7) * 0.5 + 100.0
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float64)
    out = []
    for i in range(frames):
        img = bilinear(base, xs - 0.03 * i, ys - 0.02 * i)
        if i >= 2:
            x0, y0 = min(w // 5 + 3 * (i - 2), w - mover), h // 3
            img[y0:y0 + mover, x0:x0 + mover] = tex
        img = img + (uniform(seed, 300 + i, w * h) * 6.0 - 3.0).reshape(h, w)
        if jump_at is not None and i >= jump_at:
            img = img + 40.0
        out.append(to_u8(img))
    return out


def framegen_pair(kind: str, w: int, h: int, shift, seed: int):
    """A frame pair for frame generation: "pair", a warped pair (a global shift and a smooth field of 0.5 px); "scene",
    a scene change (the same picture 110 grey brighter and inverted)."""
    if kind == "scene":
        f0 = noise_frame(w, h, seed)
        return f0, (255 - np.minimum(f0.astype(np.int32) + 110, 255)).astype(np.uint8)
    f0, f1, _, _ = warp_pair(w, h, shift, 0.5, seed=seed)
    return f0, f1


def build_frame(kind: str, w: int, h: int, seed: int) -> np.ndarray:
    """A frame for tk_build's input steps: "warp", a blurred-noise scene; "low", the same squeezed into grey 100 .. 140
    (what the contrast stretch is for); "flat", one grey level (no range to stretch); "dark", the scene scaled into
    0 .. 60 with a black corner (minimum 0)."""
    if kind == "flat":
        return np.full((h, w), 77, np.uint8)
    f = noise_frame(w, h, seed)
    if kind == "low":
        return (100 + (f.astype(np.int32) * 40) // 255).astype(np.uint8)
    if kind == "dark":
        d = (f.astype(np.int32) * 60 // 255).astype(np.uint8)
        d[: h // 8, : w // 8] = 0
        return d
    return f


def seeded_shift(seed: int, stream: int, reach: float = 12.0):
    u = uniform(seed, 100 + stream, 2)
    return (float(-reach + 2 * reach * u[0]), float(-reach + 2 * reach * u[1]))


def ncc_templates(frame: np.ndarray, size: int, count: int, seed: int, blank_share: float = 0.1):
    """count templates of size x size (uint8) and their true corners (x, y); entries of `blank` are near-blank."""
    h, w = frame.shape
    u = uniform(seed, 200 + size, count * 5).reshape(count, 5)
    xs = (2 + np.floor(u[:, 0] * (w - size - 6))).astype(np.int64)
    ys = (2 + np.floor(u[:, 1] * (h - size - 6))).astype(np.int64)
    gain = 0.8 + 0.4 * u[:, 2]
    off = -20.0 + 40.0 * u[:, 3]
    nblank = int(round(count * blank_share))
    blank = np.zeros(count, bool)
    blank[np.argsort(u[:, 4], kind="stable")[:nblank]] = True
    out = np.zeros((count, size, size), np.uint8)
    for i in range(count):
        g = uniform(seed, 300 + 1000 * size + i, size * size * 12).reshape(12, size, size).sum(axis=0) - 6.0
        if blank[i]:
            level = 40.0 + 170.0 * u[i, 2]
            flat = level + 1.5 * (uniform(seed, 500 + 1000 * size + i, size * size).reshape(size, size) * 2.0 - 1.0)
            out[i] = to_u8(flat)
        else:
            patch = frame[ys[i]:ys[i] + size, xs[i]:xs[i] + size].astype(np.float64)
            out[i] = to_u8(patch * gain[i] + off[i] + 3.0 * g)
    return out, xs, ys, blank


# The benchmark configurations (sizes, grids and LK settings).
CONFIG_640 = dict(w=640, h=480, levels=3, cell_w=16, cell_h=16, shift=(1.7, -0.8), seed=1)
CONFIG_1080 = dict(w=1920, h=1080, levels=4, cell_w=16, cell_h=8, seed=2)
LK_DEFAULTS = dict(patch_w=21, patch_h=21, max_iter=10, eps=0.01, min_eig=0.1, max_residual=25.0, fb_max=0.5)
