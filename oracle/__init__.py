"""CPU oracle for the Anime4KCPP upscaling path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use this package, and only to compare results against or as the
timed CPU baseline.  The product library (``anime4kcpp_gb300``) never imports it.

Two back ends:

* ``liboracle.so`` -- this project's C restatement of the reference CPU path
  (``acoracle.c``; FP32 in the reference's Generic operation order plus an FP64
  twin).  Built by ``make -C oracle`` on any host.
* ``_ref/libacref.so`` -- the reference's own CPU processor compiled from its
  sources by ``make -C oracle ref``.  Exists only where the reference sources
  were present at build time; never shipped as product.

The pipeline function :func:`process` restates ``Processor::process``
(core/src/processor/Processor.cpp:199-276) on top of the C primitives.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
WEIGHTS_BLOB = os.path.join(ROOT, "anime4kcpp_gb300", "weights", "acnet_legacy.bin")
ACNET8_BLOB = os.path.join(ROOT, "anime4kcpp_gb300", "weights", "acnet8.bin")
F3_BLOB = os.path.join(ROOT, "anime4kcpp_gb300", "weights", "artcnn_fsrcnnx.bin")

U8, U16, F32 = 0x001, 0x002, 0x204
_TYPE_OF = {np.dtype(np.uint8): U8, np.dtype(np.uint16): U16, np.dtype(np.float32): F32}
_DTYPE_OF = {U8: np.uint8, U16: np.uint16, F32: np.float32}

RESIZE_POINT, RESIZE_CATMULL_ROM, RESIZE_BILINEAR = 0, 1, 16
ARNET_SEED_BASE = 0x41524E6574000000

_lock = threading.Lock()
_lib = None
_ref = None


def build(force=False):
    """Compile liboracle.so with make (fast; a single C file)."""
    so = os.path.join(HERE, "liboracle.so")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(os.path.join(HERE, "acoracle.c")):
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return so


def lib():
    global _lib
    with _lock:
        if _lib is None:
            so = build()
            L = ctypes.CDLL(so)
            vp, i, f, d, fp, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p
            L.orc_acnet_legacy_x2.argtypes = [vp, i, i, i, i, vp, i, fp, fp, i]
            L.orc_acnet_legacy_x2_simd4.argtypes = [vp, i, i, i, i, vp, i, fp, fp, i]
            L.orc_acnet_legacy_x2_f64.argtypes = [vp, i, i, i, i, dp, fp, fp, i]
            L.orc_arnet_x2.argtypes = [vp, i, i, i, i, vp, i, fp, fp, fp, i, i]
            L.orc_arnet_x2_f64.argtypes = [vp, i, i, i, i, dp, fp, fp, fp, i, i]
            L.orc_acnet8_x2.argtypes = [vp, i, i, i, i, vp, i, fp, fp, fp, i, i]
            L.orc_acnet8_x2_f64.argtypes = [vp, i, i, i, i, dp, fp, fp, fp, i, i]
            L.orc_f3_x2_f64.argtypes = [vp, i, i, i, i, dp, fp, fp, fp, i, i, i, i]
            L.orc_artcnn_x2.argtypes = [vp, i, i, i, i, vp, i, fp, fp, i, i, i]
            L.orc_fsrcnnx_x2.argtypes = [vp, i, i, i, i, vp, i, fp, fp, fp, i, i, i]
            L.orc_rgb2yuv.argtypes = [vp, i, i, i, i, i, vp, i, vp, i]
            L.orc_yuv2rgb.argtypes = [vp, i, vp, i, i, i, i, i, vp, i]
            L.orc_resize.argtypes = [vp, i, i, i, i, i, vp, i, i, i, i]
            L.orc_resize_mt.argtypes = [vp, i, i, i, i, i, vp, i, i, i, i, i]
            L.orc_resize_coeffs.argtypes = [i, i, i, vp, vp, i]
            L.orc_arnet_synth.argtypes = [i, ctypes.c_uint64, fp, fp, fp]
            for fn in ("orc_acnet_legacy_x2", "orc_acnet_legacy_x2_simd4", "orc_acnet_legacy_x2_f64", "orc_arnet_x2", "orc_arnet_x2_f64",
                       "orc_acnet8_x2", "orc_acnet8_x2_f64", "orc_f3_x2_f64", "orc_artcnn_x2", "orc_fsrcnnx_x2",
                       "orc_rgb2yuv", "orc_yuv2rgb", "orc_resize", "orc_resize_mt", "orc_resize_coeffs", "orc_arnet_synth"):
                getattr(L, fn).restype = ctypes.c_int
            _lib = L
    return _lib


def ref_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libacref.so"))


def ref():
    """The reference's own CPU processor (only where it was compiled)."""
    global _ref
    with _lock:
        if _ref is None:
            R = ctypes.CDLL(os.path.join(HERE, "_ref", "libacref.so"))
            vp, i = ctypes.c_void_p, ctypes.c_int
            R.acref_process.argtypes = [ctypes.c_char_p, i, vp, i, i, i, i, i, vp, i, i, i, ctypes.c_double]
            R.acref_process.restype = i
            R.acref_name.argtypes = [ctypes.c_char_p, i]
            R.acref_name.restype = ctypes.c_char_p
            R.acref_rgb2yuv.argtypes = [vp, i, i, i, i, i, vp, i, vp, i]
            R.acref_yuv2rgb.argtypes = [vp, i, vp, i, i, i, i, i, vp, i]
            _ref = R
    return _ref


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _plane(a):
    a = np.ascontiguousarray(a)
    if a.dtype not in _TYPE_OF:
        raise TypeError("unsupported dtype %s" % a.dtype)
    return a


# ------------------------------------------------------------------ models

def parse_model(name):
    """Model string -> (family, variant) following Processor.cpp:26-187.
    Returns ("acnet_legacy", idx 0..4) with 0=GAN, 1..4=HDN0..3,
    ("acnet8", (blocks, kind)) or ("arnet", (blocks, kind)) with kind 0
    normal, 1 HDN, 2 Box, 3 Box-HDN, ("artcnn", (F, kind 0 normal / 1 DN /
    2 DS)) or ("fsrcnnx", (F, kind 0 normal / 1 DistortPlus))."""
    s = (name or "").lower()
    if "arnet" in s:
        box = "box" in s
        hdn = "hdn" in s
        blocks = 8
        for tag, b in (("b8", 8), ("b16", 16), ("b32", 32), ("b64", 64)):
            if tag in s:
                blocks = b
                break
        kind = (2 if box else 0) + (1 if hdn else 0)
        return "arnet", (blocks, kind)
    if "acnet" in s and "legacy" in s:
        idx = 0
        if "hdn" in s:
            idx = 1
            for ch in s:
                if ch in "0123":
                    idx = 1 + int(ch)
                    break
        return "acnet_legacy", idx
    if "fsrcnnx" in s:
        # Processor.cpp:40-55
        return "fsrcnnx", (16 if "f16" in s else 8, 1 if ("distort" in s or "dp" in s) else 0)
    if "artcnn" in s:
        # Processor.cpp:56-74
        return "artcnn", (32 if "f32" in s else 16, 1 if "dn" in s else (2 if "ds" in s else 0))
    if "acnet" in s:
        # Processor.cpp:146-184: b4, then b8, then b18; B8 by default.
        blocks = 8
        for tag, b in (("b4", 4), ("b8", 8), ("b18", 18)):
            if tag in s:
                blocks = b
                break
        return "acnet8", (blocks, (2 if "box" in s else 0) + (1 if "hdn" in s else 0))
    return "acnet_legacy", 0


_weights_cache = {}


def acnet_legacy_weights(variant):
    """(kernels[4712], biases[72]) float32 for variant 0=GAN, 1..4=HDN0..3."""
    if "acnet" not in _weights_cache:
        raw = open(WEIGHTS_BLOB, "rb").read()
        assert raw[:8] == b"ACGBW001"
        n, nk, nb = np.frombuffer(raw[8:20], dtype="<u4")
        arr = np.frombuffer(raw[20:], dtype="<f4").reshape(int(n), int(nk + nb))
        _weights_cache["acnet"] = (arr, int(nk))
    arr, nk = _weights_cache["acnet"]
    return np.ascontiguousarray(arr[variant, :nk]), np.ascontiguousarray(arr[variant, nk:])


def arnet_weights(blocks, kind):
    key = ("arnet", blocks, kind)
    if key not in _weights_cache:
        nconv = 2 * blocks
        k = np.zeros(72 + 576 * nconv + 64 + 288, np.float32)
        b = np.zeros(8 + 8 * (nconv + 1) + 4, np.float32)
        a = np.zeros(8 * (blocks + 1), np.float32)
        rc = lib().orc_arnet_synth(blocks, ARNET_SEED_BASE + 16 * blocks + kind, _p(k), _p(b), _p(a))
        assert rc == 0
        _weights_cache[key] = (k, b, a)
    return _weights_cache[key]


def acnet8_weights(blocks, kind):
    """(kernels, biases, alphas) float32 of the trained ACNet<8> variant
    (blocks 4/8/18; kind 0 normal, 1 HDN, 2 Box, 3 Box-HDN), read from the
    blob extracted from the reference's ACNet.p."""
    if "acnet8" not in _weights_cache:
        raw = open(ACNET8_BLOB, "rb").read()
        assert raw[:8] == b"ACGBW8F1"
        n = int(np.frombuffer(raw[8:12], dtype="<u4")[0])
        at, table = 12, {}
        for v in range(n):
            b, nk, nb, na = (int(x) for x in np.frombuffer(raw[at:at + 16], dtype="<u4"))
            f = np.frombuffer(raw[at + 16:at + 16 + 4 * (nk + nb + na)], dtype="<f4")
            table[(b, v % 4)] = (np.ascontiguousarray(f[:nk]), np.ascontiguousarray(f[nk:nk + nb]),
                                 np.ascontiguousarray(f[nk + nb:]))
            at += 16 + 4 * (nk + nb + na)
        _weights_cache["acnet8"] = table
    return _weights_cache["acnet8"][(blocks, kind)]


def f3_weights(family, F, kind):
    """(kernels, biases, alphas) float32 of a trained ArtCNN ("artcnn") or
    FSRCNNX ("fsrcnnx") variant, read from the blob extracted from the
    reference's ArtCNN.p / FSRCNNX.p (4 blocks each)."""
    if "f3" not in _weights_cache:
        raw = open(F3_BLOB, "rb").read()
        assert raw[:8] == b"ACGBW9F1"
        n = int(np.frombuffer(raw[8:12], dtype="<u4")[0])
        at, table = 12, {}
        for _ in range(n):
            fam, f, blocks, k, nk, nb, na = (int(x) for x in np.frombuffer(raw[at:at + 28], dtype="<u4"))
            v = np.frombuffer(raw[at + 28:at + 28 + 4 * (nk + nb + na)], dtype="<f4")
            table[(fam, f, k)] = (np.ascontiguousarray(v[:nk]), np.ascontiguousarray(v[nk:nk + nb]),
                                  np.ascontiguousarray(v[nk + nb:]) if na else np.zeros(1, np.float32))
            at += 28 + 4 * (nk + nb + na)
        _weights_cache["f3"] = table
    return _weights_cache["f3"][(1 if family == "artcnn" else 2, F, kind)]


# --------------------------------------------------------------- primitives

def luma_x2(y, model, threads=0, f64=False, order="generic"):
    """One x2 luma pass of ``model`` over a 2-D plane (u8/u16/f32).  ``order``
    "neon" runs ACNetLegacy in the operation order of the reference's NEON
    backend (4-lane partial sums; the CPU baseline on aarch64 hosts)."""
    y = _plane(y)
    h, w = y.shape
    t = _TYPE_OF[y.dtype]
    threads = threads or os.cpu_count() or 1
    fam, var = parse_model(model)
    if f64:
        out = np.empty((2 * h, 2 * w), np.float64)
        if fam == "acnet_legacy":
            k, b = acnet_legacy_weights(var)
            rc = lib().orc_acnet_legacy_x2_f64(_p(y), w, h, y.strides[0], t, _p(out), _p(k), _p(b), threads)
        elif fam == "acnet8":
            k, b, a = acnet8_weights(*var)
            rc = lib().orc_acnet8_x2_f64(_p(y), w, h, y.strides[0], t, _p(out), _p(k), _p(b), _p(a), var[0], threads)
        elif fam in ("artcnn", "fsrcnnx"):
            k, b, a = f3_weights(fam, *var)
            rc = lib().orc_f3_x2_f64(_p(y), w, h, y.strides[0], t, _p(out), _p(k), _p(b), _p(a),
                                     1 if fam == "artcnn" else 2, var[0], 4, threads)
        else:
            k, b, a = arnet_weights(*var)
            rc = lib().orc_arnet_x2_f64(_p(y), w, h, y.strides[0], t, _p(out), _p(k), _p(b), _p(a), var[0], threads)
    else:
        out = np.empty((2 * h, 2 * w), y.dtype)
        if fam == "acnet_legacy":
            k, b = acnet_legacy_weights(var)
            fn = lib().orc_acnet_legacy_x2_simd4 if order == "neon" else lib().orc_acnet_legacy_x2
            rc = fn(_p(y), w, h, y.strides[0], t, _p(out), out.strides[0], _p(k), _p(b), threads)
        elif fam == "acnet8":
            k, b, a = acnet8_weights(*var)
            rc = lib().orc_acnet8_x2(_p(y), w, h, y.strides[0], t, _p(out), out.strides[0], _p(k), _p(b), _p(a), var[0],
                                     threads)
        elif fam == "artcnn":
            k, b, _ = f3_weights(fam, *var)
            rc = lib().orc_artcnn_x2(_p(y), w, h, y.strides[0], t, _p(out), out.strides[0], _p(k), _p(b), var[0], 4, threads)
        elif fam == "fsrcnnx":
            k, b, a = f3_weights(fam, *var)
            rc = lib().orc_fsrcnnx_x2(_p(y), w, h, y.strides[0], t, _p(out), out.strides[0], _p(k), _p(b), _p(a), var[0], 4,
                                      threads)
        else:
            k, b, a = arnet_weights(*var)
            rc = lib().orc_arnet_x2(_p(y), w, h, y.strides[0], t, _p(out), out.strides[0], _p(k), _p(b), _p(a), var[0], threads)
    if rc != 0:
        raise RuntimeError("oracle luma pass failed: %d" % rc)
    return out


def rgb2yuv(img):
    img = _plane(img)
    h, w, c = img.shape
    y = np.empty((h, w), img.dtype)
    uv = np.empty((h, w, 3 if c == 4 else 2), img.dtype)
    rc = lib().orc_rgb2yuv(_p(img), w, h, c, img.strides[0], _TYPE_OF[img.dtype], _p(y), y.strides[0], _p(uv), uv.strides[0])
    assert rc == 0
    return y, uv


def yuv2rgb(y, uv):
    y = _plane(y)
    uv = _plane(uv)
    h, w = y.shape
    c = 4 if uv.shape[2] == 3 else 3
    out = np.empty((h, w, c), y.dtype)
    rc = lib().orc_yuv2rgb(_p(y), y.strides[0], _p(uv), uv.strides[0], w, h, c, _TYPE_OF[y.dtype], _p(out), out.strides[0])
    assert rc == 0
    return out


def resize(img, dw, dh, mode=RESIZE_CATMULL_ROM, threads=0):
    img = _plane(img)
    threads = threads or os.cpu_count() or 1
    squeeze = img.ndim == 2
    if squeeze:
        img = img[:, :, None]
    h, w, c = img.shape
    out = np.empty((dh, dw, c), img.dtype)
    rc = lib().orc_resize_mt(_p(img), w, h, c, img.strides[0], _TYPE_OF[img.dtype], _p(out), dw, dh, out.strides[0], mode, threads)
    assert rc == 0
    return out[:, :, 0] if squeeze else out


def resize_coeffs(n_in, n_out, mode=RESIZE_CATMULL_ROM, maxtaps=64):
    first = np.zeros(n_out, np.int32)
    wts = np.zeros((n_out, maxtaps), np.float32)
    lib().orc_resize_coeffs(n_in, n_out, mode, _p(first), _p(wts), maxtaps)
    return first, wts


def _ceil_log2(v):
    # Util.hpp:80-89: exponent of v plus one when the mantissa is non-zero.
    m, e = np.frexp(v)
    return int(e - 1 + (1 if m != 0.5 else 0))


# ----------------------------------------------------------------- pipeline

def process(img, factor, model, threads=0, order="generic"):
    """Restatement of Processor::process (Processor.cpp:199-276) with an empty
    dst: luma passes, luma resize by the residual factor, chroma resize by the
    full factor, colour merge.  ``img`` is (H, W) or (H, W, 3|4).  ``order``
    as for luma_x2."""
    img = _plane(img)
    power = _ceil_log2(factor) if factor > 2.0 else 1
    fxy = factor / float(1 << power)
    if img.ndim == 3 and img.shape[2] == 1:
        img = img[:, :, 0]
    if img.ndim == 2:
        out = img
        for _ in range(power):
            out = luma_x2(out, model, threads, order=order)
        if fxy != 1.0:
            out = resize(out, int(out.shape[1] * fxy), int(out.shape[0] * fxy))
        return out
    y, uv = rgb2yuv(img)
    out = y
    for _ in range(power):
        out = luma_x2(out, model, threads, order=order)
    if fxy != 1.0:
        out = resize(out, int(out.shape[1] * fxy), int(out.shape[0] * fxy))
    h, w = img.shape[:2]
    uv2 = resize(uv, int(w * factor), int(h * factor))
    return yuv2rgb(out, uv2)


def process_f64(img, model, threads=0):
    """One x2 pass of the network in FP64 over a luma plane; returns the
    unquantised, unsaturated (2H, 2W) float64 output."""
    return luma_x2(img, model, threads, f64=True)


_MAXV = {np.dtype(np.uint8): 255.0, np.dtype(np.uint16): 65535.0, np.dtype(np.float32): 1.0}


def from_float_np(v, dtype):
    """fromFloat<T> (Util.hpp:64-78) in numpy: saturate to [0, 1]; integer
    types scale by their maximum, add 0.5 and truncate; f32 is only
    saturated."""
    dtype = np.dtype(dtype)
    s = np.clip(v, 0.0, 1.0)
    if dtype == np.float32:
        return s.astype(np.float32)
    return np.floor(s * _MAXV[dtype] + 0.5).astype(dtype)


def pipeline_f64(img, model, threads=0):
    """The x2 path of Processor::process (Processor.cpp:199-276) with the luma
    network evaluated in FP64 (process_f64) and every other step as the
    reference does it: rgb2yuv quantised to the source type, chroma resized
    by the Catmull-Rom restatement, yuv2rgb.

    Returns (exact, quantised):
      exact      float64 output in units of the type's full scale (u8: /255),
                 the network's value saturated like fromFloat but not rounded,
                 the colour merge computed in FP64 on it, saturated;
      quantised  the output the reference's own path would give if its
                 network arithmetic were exact: the FP64 luma through fromFloat
                 to the source type, then yuv2rgb (the reference's rounding
                 points)."""
    img = _plane(img)
    if img.ndim == 3 and img.shape[2] == 1:
        img = img[:, :, 0]
    maxv = _MAXV[img.dtype]
    if img.ndim == 2:
        y64 = process_f64(img, model, threads)
        return np.clip(y64, 0.0, 1.0), from_float_np(y64, img.dtype)
    h, w, c = img.shape
    y, uv = rgb2yuv(img)
    y64 = process_f64(y, model, threads)
    uv2 = resize(uv, 2 * w, 2 * h, threads=threads)
    quant = yuv2rgb(from_float_np(y64, img.dtype), uv2)
    yy = np.clip(y64, 0.0, 1.0)
    u = uv2[:, :, 0].astype(np.float64) / maxv - 0.5
    v = uv2[:, :, 1].astype(np.float64) / maxv - 0.5
    rgb = np.stack([yy + 1.403 * v, yy - 0.344 * u - 0.714 * v, yy + 1.773 * u], axis=-1)
    if c == 4:
        a = uv2[:, :, 2].astype(np.float64) / maxv
        safe = np.where(a > 1e-6, a, 1.0)
        rgb = np.where((a > 1e-6)[:, :, None], rgb / safe[:, :, None], 0.0)
        rgb = np.concatenate([rgb, a[:, :, None]], axis=-1)
    return np.clip(rgb, 0.0, 1.0), quant


def error_stats(got, exact, quantised):
    """Error of a result against the FP64 oracle (pipeline_f64):

      max_abs           largest |result - exact| in full-scale units
      psnr_db           10 log10(1 / mean squared error), peak 1.0
      max_lsb           largest |result - quantised| in the type's LSB
                        (integer types; for f32 the same in units of 1e-4)
      frac_within_1lsb  share of samples with |result - quantised| <= 1 LSB
                        (f32: <= 1e-4)"""
    got = np.asarray(got)
    if got.dtype == np.float32:
        g = got.astype(np.float64)
        dq = np.abs(g - quantised.astype(np.float64)) / 1e-4
    else:
        g = got.astype(np.float64) / _MAXV[got.dtype]
        dq = np.abs(got.astype(np.int64) - quantised.astype(np.int64)).astype(np.float64)
    e = g - exact
    mse = float(np.mean(e * e))
    return {"max_abs": float(np.abs(e).max()), "psnr_db": 99.0 if mse == 0 else float(10 * np.log10(1.0 / mse)),
            "max_lsb": float(dq.max()), "frac_within_1lsb": float((dq <= 1.0).mean()), "samples": int(got.size)}


# ----------------------------------------------------- the reference itself

def ref_process(img, factor, model, arch=1):
    """Run the reference's own CPU processor (arch 1 = Generic backend,
    0 = its automatic ISA choice) with an empty dst."""
    img = _plane(img)
    squeeze = img.ndim == 2
    src = img[:, :, None] if squeeze else img
    h, w, c = src.shape
    power = _ceil_log2(factor) if factor > 2.0 else 1
    dw, dh = w, h
    for _ in range(power):
        dw, dh = dw * 2, dh * 2
    fxy = factor / float(1 << power)
    if fxy != 1.0:
        dw, dh = int(dw * fxy), int(dh * fxy)
    if c > 1:
        dw, dh = int(w * factor), int(h * factor)
    out = np.zeros((dh, dw, c), src.dtype)
    rc = ref().acref_process(model.encode(), arch, _p(src), w, h, c, src.strides[0], _TYPE_OF[src.dtype],
                             _p(out), dw, dh, out.strides[0], float(factor))
    if rc != 0:
        raise RuntimeError("reference process failed: %d" % rc)
    return out[:, :, 0] if squeeze else out
