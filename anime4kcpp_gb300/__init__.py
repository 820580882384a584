"""GB300-native backend for the Anime4KCPP CNN upscaling path.

The compute path is the native library ``libac_gb300.so`` (hand-written
sm_103a CUDA behind a C ABI that mirrors the reference's ``binding/c``).  This
module is a thin ctypes host layer that mirrors the reference's Python
binding (binding/python/src/Binding.cpp:21-62): ``Processor(type, device,
model)`` with ``process(array, factor)``, ``ok()``, ``error()``, ``name()``,
``__call__`` raising on error, and ``resize(...)``.

There is no CPU fallback: if the native library is missing, importing the
processor raises.  Build it with ``python -m anime4kcpp_gb300.build``.
"""
import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libac_gb300.so")

UINT8, UINT16, FLOAT32 = 0x001, 0x002, 0x204
_TYPE_OF = {np.dtype(np.uint8): UINT8, np.dtype(np.uint16): UINT16, np.dtype(np.float32): FLOAT32}
PRECISIONS = {"fp32": 0, "fp16": 1, "bf16": 2}

AC_SUCCESS = 0
AC_EIO, AC_EINVAL, AC_EPROCESSOR = 5, 22, 256

(RESIZE_POINT, RESIZE_CATMULL_ROM, RESIZE_MITCHELL_NETRAVALI, RESIZE_BICUBIC_0_60, RESIZE_BICUBIC_0_75,
 RESIZE_BICUBIC_0_100, RESIZE_BICUBIC_20_50, RESIZE_SOFTCUBIC50, RESIZE_SOFTCUBIC75, RESIZE_SOFTCUBIC100,
 RESIZE_LANCZOS2, RESIZE_LANCZOS3, RESIZE_LANCZOS4, RESIZE_SPLINE16, RESIZE_SPLINE36, RESIZE_SPLINE64,
 RESIZE_BILINEAR) = range(17)


class ACImage(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("channels", ctypes.c_int),
                ("stride", ctypes.c_int), ("element_type", ctypes.c_int), ("ptr", ctypes.c_void_p),
                ("hptr", ctypes.c_void_p)]


class ACProcessor(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("type", ctypes.c_char_p), ("model", ctypes.c_char_p),
                ("hptr", ctypes.c_void_p)]


class ACGB300DeviceImage(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("channels", ctypes.c_int), ("stride", ctypes.c_int), ("element_type", ctypes.c_int)]


class ACGB300HostPlane(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("width", ctypes.c_int), ("height", ctypes.c_int), ("channels", ctypes.c_int),
                ("stride", ctypes.c_int), ("element_type", ctypes.c_int)]


class ACGB300ServeJob(ctypes.Structure):
    _fields_ = [("model", ctypes.c_char_p), ("factor", ctypes.c_double), ("planes", ctypes.c_int), ("shift", ctypes.c_int),
                ("src", ACGB300HostPlane * 3), ("dst", ACGB300HostPlane * 3)]


class ACGB300ServeResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("queue_ms", ctypes.c_double), ("device_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double), ("h2d_ms", ctypes.c_double), ("compute_ms", ctypes.c_double),
                ("d2h_ms", ctypes.c_double), ("batch", ctypes.c_int), ("error", ctypes.c_char * 160)]


class ACGB300ServeStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "failed", "batches", "batched_jobs")] + \
               [(n, ctypes.c_double) for n in ("budget_bytes", "in_use_bytes", "peak_bytes", "pool_bytes")] + \
               [("device_allocs", ctypes.c_uint64)]


# Every symbol of include/ac_image.h, include/ac_processor.h and include/ac_gb300.h.
EXPORTS = (
    "ac_image_alloc", "ac_image_free", "ac_image_ref", "ac_image_unref", "ac_image_create", "ac_image_map",
    "ac_image_from", "ac_image_view", "ac_image_clone", "ac_image_to", "ac_resize", "ac_rgb2yuv", "ac_rgba2yuva",
    "ac_yuv2rgb", "ac_yuva2rgba",
    "ac_processor_alloc", "ac_processor_free", "ac_processor_ref", "ac_processor_unref", "ac_processor_create",
    "ac_processor_process", "ac_processor_ok", "ac_processor_error", "ac_processor_name", "ac_processor_type",
    "ac_processor_type_name", "ac_processor_info", "ac_processor_list_info",
    "ac_gb300_set_precision", "ac_gb300_get_precision", "ac_gb300_output_shape", "ac_gb300_process_device",
    "ac_gb300_launch_count", "ac_gb300_model_params", "ac_gb300_profile_enable", "ac_gb300_profile_collect",
    "ac_gb300_tc_selftest", "ac_gb300_wait_selftest", "ac_gb300_process_device_noalloc", "ac_gb300_process_batch_device",
    "ac_gb300_graph_replays", "ac_gb300_last_plan", "ac_gb300_debug_fail_alloc", "ac_gb300_process_yuv_device",
    "ac_gb300_server_create", "ac_gb300_server_error", "ac_gb300_server_submit", "ac_gb300_server_wait",
    "ac_gb300_server_stats", "ac_gb300_server_destroy",
)

_lock = threading.Lock()
_lib = None


def native():
    """The loaded native library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libac_gb300.so not built: run `python -m anime4kcpp_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        P, I, D, V = ctypes.POINTER, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
        pimg, pproc = P(ACImage), P(ACProcessor)
        sig = {
            "ac_image_alloc": (pimg, []), "ac_image_free": (None, [P(pimg)]), "ac_image_ref": (I, [pimg, pimg]),
            "ac_image_unref": (None, [pimg]), "ac_image_create": (I, [pimg]), "ac_image_map": (I, [pimg]),
            "ac_image_from": (I, [pimg, V]), "ac_image_view": (I, [pimg, pimg, I, I, I, I]),
            "ac_image_clone": (I, [pimg, pimg]), "ac_image_to": (I, [pimg, V, I]),
            "ac_resize": (I, [pimg, pimg, D, D, I]), "ac_rgb2yuv": (I, [pimg, pimg]),
            "ac_rgba2yuva": (I, [pimg, pimg]), "ac_yuv2rgb": (I, [pimg, pimg]), "ac_yuva2rgba": (I, [pimg, pimg]),
            "ac_processor_alloc": (pproc, []), "ac_processor_free": (None, [P(pproc)]),
            "ac_processor_ref": (I, [pproc, pproc]), "ac_processor_unref": (None, [pproc]),
            "ac_processor_create": (I, [pproc]), "ac_processor_process": (I, [pproc, pimg, pimg, D]),
            "ac_processor_ok": (I, [pproc]), "ac_processor_error": (ctypes.c_char_p, [pproc]),
            "ac_processor_name": (ctypes.c_char_p, [pproc]), "ac_processor_type": (I, [pproc]),
            "ac_processor_type_name": (ctypes.c_char_p, [pproc]), "ac_processor_info": (ctypes.c_char_p, [I]),
            "ac_processor_list_info": (ctypes.c_char_p, []),
            "ac_gb300_set_precision": (I, [pproc, I]), "ac_gb300_get_precision": (I, [pproc]),
            "ac_gb300_output_shape": (I, [I, I, I, D, P(I), P(I)]),
            "ac_gb300_process_device": (I, [pproc, P(ACGB300DeviceImage), P(ACGB300DeviceImage), D, V, I]),
            "ac_gb300_process_device_noalloc": (I, [pproc, I, P(ACGB300DeviceImage), P(ACGB300DeviceImage), V, I]),
            "ac_gb300_process_batch_device": (I, [pproc, I, P(ACGB300DeviceImage), P(ACGB300DeviceImage), D, V, I]),
            "ac_gb300_graph_replays": (ctypes.c_uint64, []),
            "ac_gb300_last_plan": (I, [pproc, P(I), P(I), P(I), P(I), P(I)]),
            "ac_gb300_debug_fail_alloc": (None, [I]),
            "ac_gb300_process_yuv_device": (I, [pproc, I, I, P(ACGB300DeviceImage), P(ACGB300DeviceImage), D, I, V, I]),
            "ac_gb300_server_create": (V, [I, I, D, I, I]),
            "ac_gb300_server_error": (ctypes.c_char_p, [V]),
            "ac_gb300_server_submit": (I, [V, P(ACGB300ServeJob), P(ctypes.c_uint64)]),
            "ac_gb300_server_wait": (I, [V, ctypes.c_uint64, D, P(ACGB300ServeResult)]),
            "ac_gb300_server_stats": (I, [V, P(ACGB300ServeStats)]),
            "ac_gb300_server_destroy": (None, [V]),
            "ac_gb300_launch_count": (ctypes.c_uint64, []),
            "ac_gb300_model_params": (I, [ctypes.c_char_p, V, I, V, I, V, I, P(I)]),
            "ac_gb300_profile_enable": (I, [pproc, I]),
            "ac_gb300_profile_collect": (I, [pproc, P(D), P(I), P(D)]),
            "ac_gb300_tc_selftest": (I, [V, I, V, I, I, I, V]),
            "ac_gb300_wait_selftest": (I, [I, P(ctypes.c_int), P(ctypes.c_double)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def _map(arr):
    """An ACImage mapping a numpy array (H, W) or (H, W, C)."""
    if arr.ndim not in (2, 3):
        raise ValueError("Incompatible dimension: expected 2 or 3.")
    if arr.dtype not in _TYPE_OF:
        raise TypeError("Incompatible type: expected uint8, uint16 or float32.")
    if arr.strides[-1] != arr.itemsize or (arr.ndim == 3 and arr.strides[1] != arr.itemsize * arr.shape[2]):
        raise ValueError("rows must be contiguous")
    img = ACImage()
    img.width = arr.shape[1]
    img.height = arr.shape[0]
    img.channels = 1 if arr.ndim == 2 else arr.shape[2]
    img.stride = arr.strides[0]
    img.element_type = _TYPE_OF[arr.dtype]
    img.ptr = arr.ctypes.data
    rc = native().ac_image_map(ctypes.byref(img))
    if rc != AC_SUCCESS:
        raise RuntimeError("ac_image_map failed: %d" % rc)
    return img


def output_shape(width, height, channels, factor):
    ow, oh = ctypes.c_int(), ctypes.c_int()
    rc = native().ac_gb300_output_shape(width, height, channels, float(factor), ctypes.byref(ow), ctypes.byref(oh))
    if rc != AC_SUCCESS:
        raise ValueError("invalid shape or factor")
    return ow.value, oh.value


class _StaticProperty:
    """A read-only attribute computed on each access, on the class and on its
    instances alike (pybind11's ``def_property_readonly_static``)."""

    def __init__(self, fget):
        self.fget = fget

    def __get__(self, obj, cls=None):
        return self.fget()


class Processor:
    """Mirror of the reference's ``pyac.core.Processor`` backed by the GB300 library."""

    CPU, OpenCL, CUDA = 0, 1, 2

    def __init__(self, type="auto", device=0, model="acnet-legacy-hdn0", precision=None):
        L = native()
        self._type_b = type.encode() if isinstance(type, str) else type
        self._model_b = model.encode() if isinstance(model, str) else model
        self._p = ACProcessor()
        self._p.device = device
        self._p.type = self._type_b
        self._p.model = self._model_b
        L.ac_processor_create(ctypes.byref(self._p))
        if precision is not None and self.ok():
            self.set_precision(precision)

    def __del__(self):
        try:
            if self._p.hptr:
                native().ac_processor_unref(ctypes.byref(self._p))
        except Exception:
            pass

    # reference binding surface ------------------------------------------------
    def ok(self):
        return native().ac_processor_ok(ctypes.byref(self._p)) == AC_SUCCESS

    def error(self):
        e = native().ac_processor_error(ctypes.byref(self._p))
        return e.decode() if e else ""

    def name(self):
        n = native().ac_processor_name(ctypes.byref(self._p))
        return n.decode() if n else ""

    def type(self):
        return native().ac_processor_type(ctypes.byref(self._p))

    def type_name(self):
        n = native().ac_processor_type_name(ctypes.byref(self._p))
        return n.decode() if n else ""

    def __str__(self):
        return self.name()

    def process(self, src, factor=2.0, dst=None):
        """Upscale a host array (H, W) or (H, W, C).  Like the reference
        binding, dst is preallocated as (int(H*factor), int(W*factor)[, C])."""
        src = np.asarray(src)
        if dst is None:
            shape = (int(src.shape[0] * factor), int(src.shape[1] * factor)) + tuple(src.shape[2:])
            dst = np.empty(shape, src.dtype)
        si, di = _map(src), _map(dst)
        native().ac_processor_process(ctypes.byref(self._p), ctypes.byref(si), ctypes.byref(di), float(factor))
        native().ac_image_unref(ctypes.byref(si))
        native().ac_image_unref(ctypes.byref(di))
        return dst

    def __call__(self, src, factor=2.0):
        out = self.process(src, factor)
        if not self.ok():
            raise RuntimeError(self.error())
        return out

    # GB300 extensions -------------------------------------------------------
    def set_precision(self, precision):
        p = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        if native().ac_gb300_set_precision(ctypes.byref(self._p), p) != AC_SUCCESS:
            raise ValueError("cannot set precision %r" % (precision,))

    def precision(self):
        v = native().ac_gb300_get_precision(ctypes.byref(self._p))
        return {0: "fp32", 1: "fp16", 2: "bf16"}.get(v, v)

    def process_device(self, src, dst, factor=2.0, stream=None, sync=True):
        """Upscale between device buffers.  ``src``/``dst`` are objects with
        ``data_ptr()``, ``shape``, ``stride()`` and ``dtype`` (torch CUDA
        tensors, (H, W) or (H, W, C), rows contiguous) or tuples
        (ptr, w, h, c, stride_bytes, element_type).  ``stream`` is a raw
        cudaStream_t (int) or None."""
        s, d = _dev(src), _dev(dst)
        rc = native().ac_gb300_process_device(ctypes.byref(self._p), ctypes.byref(s), ctypes.byref(d), float(factor),
                                              ctypes.c_void_p(stream or 0), 1 if sync else 0)
        if rc != AC_SUCCESS:
            raise RuntimeError(self.error())

    def process_batch_device(self, srcs, dsts, factor=2.0, stream=None, sync=True):
        """Upscale many device images in one call (``ac_gb300_process_batch_device``):
        ACNetLegacy x2 in the FP16/BF16 form runs each group of one channel
        count and element type as one persistent launch."""
        n = len(srcs)
        if len(dsts) != n:
            raise ValueError("srcs and dsts differ in length")
        arr = ACGB300DeviceImage * max(n, 1)
        s, d = arr(*[_dev(x) for x in srcs]), arr(*[_dev(x) for x in dsts])
        rc = native().ac_gb300_process_batch_device(ctypes.byref(self._p), n, s, d, float(factor),
                                                    ctypes.c_void_p(stream or 0), 1 if sync else 0)
        if rc != AC_SUCCESS:
            raise RuntimeError(self.error())

    def process_yuv_device(self, frames, outs, factor=2.0, shift=0, stream=None, sync=True):
        """The reference CLI's planar video recipe on device frames
        (``ac_gb300_process_yuv_device``): ``frames`` and ``outs`` are lists
        of per-frame plane tuples (Y, U, V) or (Y, UV); Y is shifted left by
        ``shift``, upscaled and shifted back, the other planes are resized to
        their out planes' sizes with Catmull-Rom."""
        if len(frames) != len(outs) or not frames:
            raise ValueError("frames and outs must be non-empty lists of equal length")
        planes = len(frames[0])
        if any(len(f) != planes for f in frames) or any(len(o) != planes for o in outs):
            raise ValueError("every frame needs the same number of planes")
        arr = ACGB300DeviceImage * (len(frames) * planes)
        s = arr(*[_dev(p) for f in frames for p in f])
        d = arr(*[_dev(p) for o in outs for p in o])
        rc = native().ac_gb300_process_yuv_device(ctypes.byref(self._p), len(frames), planes, s, d, float(factor), int(shift),
                                                  ctypes.c_void_p(stream or 0), 1 if sync else 0)
        if rc != AC_SUCCESS:
            raise RuntimeError(self.error())

    def process_device_noalloc(self, srcs, dsts, stream=None, sync=True):
        """x2 of several device images in one launch without allocating
        (``ac_gb300_process_device_noalloc``): FP16/BF16 ACNetLegacy, at most
        64 images of one channel count and element type, after one ordinary
        call in the same precision.  Returns the C status code (AC_SUCCESS,
        or an error code with the message in ``error()``)."""
        n = len(srcs)
        if len(dsts) != n:
            raise ValueError("srcs and dsts differ in length")
        arr = ACGB300DeviceImage * max(n, 1)
        s, d = arr(*[_dev(x) for x in srcs]), arr(*[_dev(x) for x in dsts])
        return native().ac_gb300_process_device_noalloc(ctypes.byref(self._p), n, s, d, ctypes.c_void_p(stream or 0),
                                                        1 if sync else 0)

    def last_plan(self):
        """The persistent tensor-core launch plan of this thread's most
        recent call (``ac_gb300_last_plan``): kernel ("quad", "pair",
        "quad-acnet8" or None), tile (w, h), CTAs per SM and fusion depth (9:
        the whole network in one launch; 5: split in two launches, the tile
        being the second launch's)."""
        k, tw, th, ps, fd = (ctypes.c_int() for _ in range(5))
        if native().ac_gb300_last_plan(ctypes.byref(self._p), ctypes.byref(k), ctypes.byref(tw), ctypes.byref(th),
                                       ctypes.byref(ps), ctypes.byref(fd)) != AC_SUCCESS:
            raise RuntimeError("no GPU processor")
        return {"kernel": {4: "quad", 3: "pair", 5: "quad-acnet8"}.get(k.value), "tile": (tw.value, th.value),
                "ctas_per_sm": ps.value, "fusion_depth": fd.value}

    def profile(self, enable=True):
        native().ac_gb300_profile_enable(ctypes.byref(self._p), 1 if enable else 0)

    def collect_profile(self):
        """(milliseconds, launches, output pixels) of the luma passes since the last collect."""
        ms, n, px = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
        if native().ac_gb300_profile_collect(ctypes.byref(self._p), ctypes.byref(ms), ctypes.byref(n), ctypes.byref(px)) != AC_SUCCESS:
            raise RuntimeError(self.error())
        return ms.value, n.value, px.value

    InfoList = _StaticProperty(lambda: (native().ac_processor_info(0).decode(), native().ac_processor_info(2).decode()))


class Server:
    """The serving loop (``ac_gb300_server_*``): jobs of mixed resolutions,
    factors, models and formats admitted by an HBM budget, batched as they
    arrive and overlapped on the device.  Host arrays given to ``submit`` are
    kept alive here until ``wait`` returns their job."""

    def __init__(self, device=0, precision="fp16", hbm_budget_gb=80.0, workers=4, max_batch=64):
        p = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self._s = native().ac_gb300_server_create(int(device), p, float(hbm_budget_gb) * 1e9, int(workers), int(max_batch))
        if not self._s:
            raise MemoryError("ac_gb300_server_create")
        err = native().ac_gb300_server_error(self._s)
        if err:
            self.close()
            raise RuntimeError(err.decode())
        self._keep = {}

    @staticmethod
    def _plane(a):
        pl = ACGB300HostPlane()
        pl.ptr = a.ctypes.data
        pl.height, pl.width = a.shape[0], a.shape[1]
        pl.channels = 1 if a.ndim == 2 else a.shape[2]
        pl.stride = a.strides[0]
        pl.element_type = _TYPE_OF[np.dtype(a.dtype)]
        return pl

    def submit(self, src, dst, model, factor=2.0, shift=0):
        """``src``/``dst``: a numpy array (one interleaved image) or a tuple of
        planes (planar YUV, Y first).  Returns a ticket."""
        src = src if isinstance(src, (tuple, list)) else (src,)
        dst = dst if isinstance(dst, (tuple, list)) else (dst,)
        if len(src) != len(dst) or not 1 <= len(src) <= 3:
            raise ValueError("src and dst need the same number of planes (1 to 3)")
        for a in tuple(src) + tuple(dst):
            if a.strides[-1] != a.itemsize or (a.ndim == 3 and a.strides[1] != a.itemsize * a.shape[2]):
                raise ValueError("planes need contiguous rows")
        job = ACGB300ServeJob()
        mb = model.encode()
        job.model, job.factor, job.planes, job.shift = mb, float(factor), len(src), int(shift)
        for i, a in enumerate(src):
            job.src[i] = self._plane(a)
        for i, a in enumerate(dst):
            job.dst[i] = self._plane(a)
        t = ctypes.c_uint64()
        if native().ac_gb300_server_submit(self._s, ctypes.byref(job), ctypes.byref(t)) != AC_SUCCESS:
            raise RuntimeError("submit failed")
        self._keep[t.value] = (src, dst)
        return t.value

    def wait(self, ticket, timeout=120.0):
        r = ACGB300ServeResult()
        rc = native().ac_gb300_server_wait(self._s, ctypes.c_uint64(ticket), float(timeout), ctypes.byref(r))
        if rc == 1:
            raise TimeoutError("job %d not done after %.1f s" % (ticket, timeout))
        if rc != AC_SUCCESS:
            raise RuntimeError("wait failed")
        self._keep.pop(ticket, None)
        return {"status": r.status, "queue_ms": r.queue_ms, "device_ms": r.device_ms, "latency_ms": r.latency_ms,
                "h2d_ms": r.h2d_ms, "compute_ms": r.compute_ms, "d2h_ms": r.d2h_ms, "batch": r.batch,
                "error": r.error.decode()}

    def stats(self):
        st = ACGB300ServeStats()
        native().ac_gb300_server_stats(self._s, ctypes.byref(st))
        return {n: getattr(st, n) for n, _ in ACGB300ServeStats._fields_}

    def close(self):
        if getattr(self, "_s", None):
            native().ac_gb300_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def debug_fail_alloc(nth):
    """Arm the nth next device allocation of the library to fail (0 disarms)."""
    native().ac_gb300_debug_fail_alloc(int(nth))


def graph_replays():
    """Batched launches replayed from captured CUDA graphs in this process."""
    return int(native().ac_gb300_graph_replays())


def _dev(t):
    img = ACGB300DeviceImage()
    if isinstance(t, tuple):
        img.ptr, img.width, img.height, img.channels, img.stride, img.element_type = t
        return img
    import torch  # device buffers come from torch; plumbing only
    types = {torch.uint8: UINT8, torch.uint16: UINT16, torch.float32: FLOAT32}
    if t.dim() not in (2, 3) or t.stride(-1) != 1:
        raise ValueError("expected a (H, W) or (H, W, C) tensor with contiguous rows")
    img.ptr = t.data_ptr()
    img.height, img.width = t.shape[0], t.shape[1]
    img.channels = 1 if t.dim() == 2 else t.shape[2]
    img.stride = t.stride(0) * t.element_size()
    img.element_type = types[t.dtype]
    return img


def resize(src, dsize=None, fx=0.0, fy=0.0, mode=RESIZE_BILINEAR):
    """Mirror of ``pyac.core.resize`` (binding/python/src/Binding.cpp:83-111), on the GPU."""
    src = np.asarray(src)
    dh, dw = int(src.shape[0] * fy), int(src.shape[1] * fx)
    if dsize is not None:
        dw, dh = dsize
    if (dh, dw) == tuple(src.shape[:2]):
        return src.copy()
    dst = np.empty((dh, dw) + tuple(src.shape[2:]), src.dtype)
    si, di = _map(src), _map(dst)
    rc = native().ac_resize(ctypes.byref(si), ctypes.byref(di), 0.0, 0.0, int(mode))
    out_ptr = di.ptr
    native().ac_image_unref(ctypes.byref(si))
    native().ac_image_unref(ctypes.byref(di))
    if rc != AC_SUCCESS:
        raise RuntimeError("resize failed: %d" % rc)
    if out_ptr != dst.ctypes.data:
        raise RuntimeError("resize did not write into the destination buffer")
    return dst


def tc_selftest(x, b, shift, bf16=False):
    """Tensor-core self-test: x uint16 [px, 8], b uint16 [16, k]; returns (status, d[128, 16])."""
    x = np.ascontiguousarray(x, np.uint16)
    b = np.ascontiguousarray(b, np.uint16)
    d = np.zeros((128, 16), np.float32)
    rc = native().ac_gb300_tc_selftest(x.ctypes.data, x.shape[0], b.ctypes.data, b.shape[1], int(shift), 1 if bf16 else 0,
                                       d.ctypes.data)
    return rc, d


def wait_selftest(limit_ms=50):
    """The kernels' bounded wait on a phase nothing completes: (rc, status, elapsed_ms)."""
    st, el = ctypes.c_int(0), ctypes.c_double(0.0)
    rc = native().ac_gb300_wait_selftest(int(limit_ms), ctypes.byref(st), ctypes.byref(el))
    return rc, st.value, el.value


def launch_count():
    return int(native().ac_gb300_launch_count())


def model_params(model):
    """(kernels, biases, alphas) float32 arrays of a model, as the library holds them."""
    L = native()
    counts = (ctypes.c_int * 3)()
    if L.ac_gb300_model_params(model.encode(), None, 0, None, 0, None, 0, counts) != AC_SUCCESS:
        raise ValueError("unknown model %r" % model)
    k = np.zeros(counts[0], np.float32)
    b = np.zeros(counts[1], np.float32)
    a = np.zeros(max(counts[2], 1), np.float32)
    rc = L.ac_gb300_model_params(model.encode(), k.ctypes.data, k.size, b.ctypes.data, b.size, a.ctypes.data, a.size, counts)
    assert rc == AC_SUCCESS
    return k, b, a[:counts[2]]
