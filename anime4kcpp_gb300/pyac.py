"""The reference Python binding's module layout over the GB300 library.

The reference builds a module ``pyac`` (binding/python/src/Binding.cpp:15-165)
with two submodules; this module offers the same names, defaults and
behaviour, so code written against it switches by changing its import::

    from anime4kcpp_gb300 import pyac
    p = pyac.core.Processor("cuda", 0, "acnet-f8b8-hdn")
    out = p(img)                      # raises on error, like the reference
    small = pyac.core.resize(out, None, 0.5, 0.5, pyac.core.RESIZE_CATMULL_ROM)

``core``: ``Processor(type="auto", device=0, model="acnet-f8b8-hdn")`` with
``process(src, factor=2.0)``, ``__call__``, ``ok``, ``error``, ``name``,
``__str__``, ``InfoList`` and the ``CPU`` / ``OpenCL`` / ``CUDA`` constants;
``resize(src, dsize, fx=0.0, fy=0.0, mode=RESIZE_BILINEAR)``; the
``ResizeModes`` enum, its values also exported on ``core``.  ``specs``:
``ModelList`` (name, description, parameter_count, version, author, homepage
per model string the reference lists) and ``ProcessorList``.

Not provided: ``core.imread`` / ``core.imwrite`` and ``ImreadModes`` (image
file I/O is outside the upscaling path), and float16 arrays (the C ABI's
element types are u8, u16 and f32).
"""
import enum
import types

from . import Processor as _Processor
from . import model_params as _model_params
from . import resize as _resize
from . import (RESIZE_BICUBIC_0_60, RESIZE_BICUBIC_0_75, RESIZE_BICUBIC_0_100, RESIZE_BICUBIC_20_50, RESIZE_BILINEAR,
               RESIZE_CATMULL_ROM, RESIZE_LANCZOS2, RESIZE_LANCZOS3, RESIZE_LANCZOS4, RESIZE_MITCHELL_NETRAVALI,
               RESIZE_POINT, RESIZE_SOFTCUBIC50, RESIZE_SOFTCUBIC75, RESIZE_SOFTCUBIC100, RESIZE_SPLINE16, RESIZE_SPLINE36,
               RESIZE_SPLINE64)


class ResizeModes(enum.IntEnum):
    RESIZE_POINT = RESIZE_POINT
    RESIZE_CATMULL_ROM = RESIZE_CATMULL_ROM
    RESIZE_MITCHELL_NETRAVALI = RESIZE_MITCHELL_NETRAVALI
    RESIZE_BICUBIC_0_60 = RESIZE_BICUBIC_0_60
    RESIZE_BICUBIC_0_75 = RESIZE_BICUBIC_0_75
    RESIZE_BICUBIC_0_100 = RESIZE_BICUBIC_0_100
    RESIZE_BICUBIC_20_50 = RESIZE_BICUBIC_20_50
    RESIZE_SOFTCUBIC50 = RESIZE_SOFTCUBIC50
    RESIZE_SOFTCUBIC75 = RESIZE_SOFTCUBIC75
    RESIZE_SOFTCUBIC100 = RESIZE_SOFTCUBIC100
    RESIZE_LANCZOS2 = RESIZE_LANCZOS2
    RESIZE_LANCZOS3 = RESIZE_LANCZOS3
    RESIZE_LANCZOS4 = RESIZE_LANCZOS4
    RESIZE_SPLINE16 = RESIZE_SPLINE16
    RESIZE_SPLINE36 = RESIZE_SPLINE36
    RESIZE_SPLINE64 = RESIZE_SPLINE64
    RESIZE_BILINEAR = RESIZE_BILINEAR


class Processor(_Processor):
    """``pyac.core.Processor`` (Binding.cpp:49-79): created with the
    reference's defaults; ``process`` returns a new array of
    (int(H * factor), int(W * factor)[, C]); calling the processor raises
    RuntimeError with ``error()`` when the call failed."""

    def __init__(self, type="auto", device=0, model="acnet-f8b8-hdn"):
        super().__init__(type, device, model)

    def process(self, src, factor=2.0):
        return super().process(src, factor)

    def __str__(self):
        return self.name()


def resize(src, dsize, fx=0.0, fy=0.0, mode=ResizeModes.RESIZE_BILINEAR):
    """``pyac.core.resize`` (Binding.cpp:99-131): dsize (width, height) or
    None with the factors fx, fy."""
    return _resize(src, dsize, fx, fy, int(mode))


def _describe(name):
    """A short description of a model string, written for this library."""
    parts = name.split("-")
    if name.startswith("acnet-legacy"):
        return "ACNetLegacy: 8 channels, nine 3x3 layers, 2x2 transposed-conv upscale (%s weights)." % parts[2].upper()
    if name.startswith("acnet-f8"):
        extra = [t for t in parts[2:]]
        return "ACNet<8>, %s blocks, PReLU, pixel-shuffle tail with the nearest input added%s." % (
            parts[1][3:], (" (" + ", ".join(extra) + " training)") if extra else "")
    if name.startswith("arnet"):
        extra = [t for t in parts[2:]]
        return ("ARNet<8>, %s residual blocks%s (this library carries seeded parameters of the trained models' shapes: "
                "the trained ones are not distributed with the reference's source)." % (
                    parts[1][3:], (" (" + ", ".join(extra) + " training)") if extra else ""))
    if name.startswith("artcnn"):
        return "ArtCNN C4F%s%s: 3x3 layers of %s channels, pixel-shuffle upscale." % (
            parts[1][3:], (" " + parts[2].upper()) if len(parts) > 2 else "", parts[1][3:])
    return "FSRCNNX F%s B4%s: 5x5 head, 3x3 layers with PReLU, 1x1 tail, pixel-shuffle upscale." % (
        parts[1][1:parts[1].index("b")], " DistortPlus" if "distort" in name else "")


# The model strings the reference lists (core/include/AC/Specs.hpp ModelList).
_MODEL_NAMES = (
    ["acnet-legacy-gan"] + ["acnet-legacy-hdn%d" % i for i in range(4)] +
    ["acnet-f8b%d%s" % (b, t) for b in (4, 8, 18) for t in ("", "-hdn", "-box", "-box-hdn")] +
    ["arnet-f8b%d%s" % (b, t) for b in (8, 16, 32, 64) for t in ("", "-hdn", "-box", "-box-hdn")] +
    ["artcnn-c4f%d%s" % (f, t) for f in (16, 32) for t in ("", "-dn", "-ds")] +
    ["fsrcnnx-f%db4%s" % (f, t) for f in (8, 16) for t in ("", "-distort-plus")])


# Provenance of the third-party trained models whose parameters this library
# carries (version, author, homepage), as the reference's list states it.
_ARTCNN = ("v1.6.2", "Artoriuz", "https://github.com/Artoriuz/ArtCNN")
_FSRCNNX = ("v1.1", "igv", "https://github.com/igv/FSRCNN-TensorFlow")
_FSRCNNX_DP = ("v1.3_distort_plus", "nessotrin", "https://github.com/nessotrin/FSRCNN-TensorFlow")


def _provenance(name):
    if name.startswith("artcnn"):
        return _ARTCNN
    if name.startswith("fsrcnnx"):
        return _FSRCNNX_DP if name.endswith("distort-plus") else _FSRCNNX
    return (None, None, None)


def _model_list():
    out = []
    for name in _MODEL_NAMES:
        k, b, a = _model_params(name)
        version, author, homepage = _provenance(name)
        out.append({"name": name, "description": _describe(name), "parameter_count": int(k.size + b.size + a.size),
                    "version": version, "author": author, "homepage": homepage})
    return tuple(out)


core = types.ModuleType("pyac.core", "Processor, resize and resize modes (the reference's pyac.core).")
core.Processor = Processor
core.resize = resize
core.ResizeModes = ResizeModes
for _m in ResizeModes:
    setattr(core, _m.name, _m)

specs = types.ModuleType("pyac.specs", "Model and processor lists (the reference's pyac.specs).")
specs.ModelList = _model_list()
specs.ProcessorList = ({"name": "cuda", "description": "GB300 (sm_103a) backend: tcgen05 tensor-core and FP32 forms."},)
