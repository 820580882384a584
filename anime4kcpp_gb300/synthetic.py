"""Seeded synthetic images for tests and benchmarks.

No public dataset is attached to the workloads this backend is measured on,
so inputs are generated: a Voronoi partition of the canvas into cells of
piecewise-constant colour, 1-px dark cell outlines, a Gaussian blur
(sigma 0.7) and additive Gaussian noise, clipped to the element type.  The
same generator produces RGB u8, 10-bit-in-u16 YUV 4:2:0 frames and f32 luma.
"""
import numpy as np


def _labels(h, w, centres, ox=0, oy=0):
    """Index of the nearest centre for every pixel (brute force in row bands)."""
    cy = centres[:, 0].astype(np.float32)
    cx = centres[:, 1].astype(np.float32)
    xs = (np.arange(w, dtype=np.float32) + ox)[None, :, None]
    out = np.empty((h, w), np.int32)
    band = max(1, (1 << 22) // max(1, w * len(centres)))
    for y0 in range(0, h, band):
        y1 = min(h, y0 + band)
        ys = (np.arange(y0, y1, dtype=np.float32) + oy)[:, None, None]
        d = (ys - cy[None, None, :]) ** 2 + (xs - cx[None, None, :]) ** 2
        out[y0:y1] = np.argmin(d, axis=2)
    return out


def _blur(img, sigma):
    """Separable Gaussian blur, radius 2, clamped edges."""
    r = 2
    t = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (t / sigma) ** 2)
    k /= k.sum()
    pad = np.pad(img, ((r, r), (r, r)) + ((0, 0),) * (img.ndim - 2), mode="edge")
    tmp = sum(k[i] * pad[:, i:i + img.shape[1]] for i in range(2 * r + 1))
    return sum(k[i] * tmp[i:i + img.shape[0]] for i in range(2 * r + 1))


def voronoi_float(h, w, cells, seed, channels=3, ox=0, oy=0, canvas=None):
    """Float image in [0, 1] (before noise): Voronoi cells + dark outlines + blur.

    ``canvas`` = (H, W) of the full canvas whose cell centres are drawn; with
    ``ox``/``oy`` a window of it is rendered (used for translated frames)."""
    rng = np.random.default_rng(seed)
    ch, cw = canvas if canvas else (h, w)
    centres = np.stack([rng.uniform(0, ch, cells), rng.uniform(0, cw, cells)], axis=1)
    colours = rng.uniform(0.08, 1.0, size=(cells, channels))
    lab = _labels(h + 1, w + 1, centres, ox, oy)
    edge = (lab[:-1, :-1] != lab[:-1, 1:]) | (lab[:-1, :-1] != lab[1:, :-1])
    img = colours[lab[:-1, :-1]]
    img[edge] = 0.04
    return _blur(img, 0.7)


def _finish(img, dtype, noise_lsb, rng, maxval):
    img = img * maxval + rng.normal(0.0, noise_lsb, size=img.shape)
    if np.dtype(dtype) == np.float32:
        return np.clip(img / maxval, 0.0, 1.0).astype(np.float32)
    return np.clip(np.rint(img), 0, maxval).astype(dtype)


def rgb_u8(h, w, cells=64, seed=0, noise=2.0, alpha=False):
    """H x W x 3 (or 4) u8 image."""
    img = voronoi_float(h, w, cells, seed, channels=3)
    out = _finish(img, np.uint8, noise, np.random.default_rng(seed + 1), 255.0)
    if alpha:
        a = np.clip(_blur(voronoi_float(h, w, 16, seed + 7, channels=1), 0.7) * 255.0 + 40, 0, 255)
        out = np.concatenate([out, np.rint(a).astype(np.uint8)], axis=2)
    return out


def luma(h, w, dtype=np.uint8, cells=64, seed=0, noise=2.0, bits=None):
    """H x W single-channel plane of u8 / u16 / f32.  ``bits`` limits the
    range of integer types (10-bit content in u16 uses bits=10)."""
    dtype = np.dtype(dtype)
    img = voronoi_float(h, w, cells, seed, channels=1)[:, :, 0]
    if dtype == np.float32:
        return _finish(img, np.float32, noise, np.random.default_rng(seed + 1), 255.0)
    maxval = float((1 << bits) - 1) if bits else float(np.iinfo(dtype).max)
    return _finish(img, dtype, noise, np.random.default_rng(seed + 1), maxval)


def f32_luma_uniform(h, w, cells=64, seed=0):
    """f32 luma with per-cell values uniform in [0, 1] plus the same outline
    structure and a 2-LSB-of-u8 noise floor."""
    rng = np.random.default_rng(seed)
    centres = np.stack([rng.uniform(0, h, cells), rng.uniform(0, w, cells)], axis=1)
    vals = rng.uniform(0.0, 1.0, size=cells)
    lab = _labels(h + 1, w + 1, centres)
    edge = (lab[:-1, :-1] != lab[:-1, 1:]) | (lab[:-1, :-1] != lab[1:, :-1])
    img = vals[lab[:-1, :-1]]
    img[edge] = 0.02
    img = _blur(img, 0.7) + rng.normal(0.0, 2.0 / 255.0, size=img.shape)
    return np.clip(img, 0.0, 1.0).astype(np.float32)


def yuv420_u16_frames(n, h, w, cells=64, seed=0, shift_px=3, noise=4.0, bits=10):
    """n frames of 10-bit content stored LSB-aligned in u16, YUV 4:2:0 planar:
    a canvas translated ``shift_px`` per frame.  Returns (Y[n,h,w], UV[n,h/2,w/2,2])."""
    ch, cw = h, w + shift_px * n
    maxval = float((1 << bits) - 1)
    ys, uvs = [], []
    rng = np.random.default_rng(seed + 99)
    for i in range(n):
        rgb = voronoi_float(h, w, cells, seed, channels=3, ox=shift_px * i, canvas=(ch, cw))
        r, g, b = rgb[..., 0], rgb[..., 1], rgb[..., 2]
        yy = 0.299 * r + 0.587 * g + 0.114 * b
        u = 0.564 * (b - yy) + 0.5
        v = 0.713 * (r - yy) + 0.5
        uv = np.stack([u, v], axis=2)
        uv = 0.25 * (uv[0::2, 0::2] + uv[1::2, 0::2] + uv[0::2, 1::2] + uv[1::2, 1::2])
        ys.append(_finish(yy, np.uint16, noise, rng, maxval))
        uvs.append(_finish(uv, np.uint16, noise, rng, maxval))
    return np.stack(ys), np.stack(uvs)


def uneven_sizes(n=64, seed=0, wmin=256, wmax=2048, hmin=256, hmax=1536):
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(hmin, hmax + 1)), int(rng.integers(wmin, wmax + 1))) for _ in range(n)]
