"""Host-side checks of the C-ABI library that need no GPU: it loads, it
exports every entry point its headers declare, model parameters match the
oracle's, processor creation fails loudly without a GPU, shape logic."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import anime4kcpp_gb300 as ac
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from anime4kcpp_gb300 import build
    build.build()
    return ac.native()


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        for m in re.finditer(r"AC_C_API\s+[^;(]*?\b(ac_\w+)\s*\(", open(h).read()):
            names.add(m.group(1))
    return names


def test_headers_declare_the_reference_binding_entry_points():
    """binding/c/include/AC/Core/{Image,Processor}.h entry points (image file
    I/O excluded) are all declared."""
    ref = {"ac_image_alloc", "ac_image_free", "ac_image_ref", "ac_image_unref", "ac_image_create", "ac_image_map",
           "ac_image_from", "ac_image_view", "ac_image_clone", "ac_image_to", "ac_resize", "ac_rgb2yuv",
           "ac_rgba2yuva", "ac_yuv2rgb", "ac_yuva2rgba", "ac_processor_alloc", "ac_processor_free",
           "ac_processor_ref", "ac_processor_unref", "ac_processor_create", "ac_processor_process",
           "ac_processor_ok", "ac_processor_error", "ac_processor_name", "ac_processor_type",
           "ac_processor_type_name", "ac_processor_info", "ac_processor_list_info"}
    assert ref <= declared_symbols()


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(ac.EXPORTS) == declared_symbols()


def test_acnet_legacy_params_match_oracle(lib):
    for name, var in [("acnet-legacy-gan", 0), ("acnet-legacy-hdn0", 1), ("acnet-legacy-hdn3", 4)]:
        k, b, a = ac.model_params(name)
        ok, ob = oracle.acnet_legacy_weights(var)
        assert np.array_equal(k, ok) and np.array_equal(b, ob) and a.size == 0


@pytest.mark.parametrize("model,blocks,kind", [("arnet-b8", 8, 0), ("arnet-hdn-b16", 16, 1), ("arnet-box-b32", 32, 2),
                                               ("arnet-box-hdn-b64", 64, 3)])
def test_arnet_synthetic_params_match_oracle(lib, model, blocks, kind):
    k, b, a = ac.model_params(model)
    ok, ob, oa = oracle.arnet_weights(blocks, kind)
    assert np.array_equal(k, ok) and np.array_equal(b, ob) and np.array_equal(a, oa)


def test_model_string_parsing(lib):
    # Processor.cpp:126-143: first digit picks the HDN level.
    for s, var in [("acnet-legacy-hdn", 1), ("ACNet-Legacy-HDN2", 3), ("acnet-legacy", 0), ("whatever", 0)]:
        k, _, _ = ac.model_params(s)
        assert np.array_equal(k, oracle.acnet_legacy_weights(var)[0])
    # every family of the reference resolves (Processor.cpp:34-184)
    for s in ("artcnn-c4f16", "fsrcnnx-f8", "arnet-b8", "acnet-f8b8"):
        assert ac.model_params(s)[0].size > 0


def test_cpu_and_opencl_types_are_refused(lib):
    for t, code in (("cpu", 0), ("opencl", 1), ("nonsense", 0)):
        p = ac.Processor(t, 0, "acnet-legacy-hdn0")
        assert not p.ok()
        assert "GB300 backend provides no" in p.error()
        assert p.type() == code


def test_artcnn_fsrcnnx_parameters_match_the_reference_blob(lib):
    """ArtCNN<16/32> (C4 x normal/DN/DS) and FSRCNNX<8/16> (B4 x normal /
    DistortPlus) resolve as the reference's model strings do and carry its
    trained parameters in the sizes of ArtCNN.hpp:28-31, FSRCNNX.hpp:28-33."""
    for F in (16, 32):
        for kind, tag in enumerate(("", "-dn", "-ds")):
            name = "artcnn-c4f%d%s" % (F, tag)
            assert oracle.parse_model(name) == ("artcnn", (F, kind))
            k, b, a = ac.model_params(name)
            assert (k.size, b.size, a.size) == (F * 9 + F * F * 9 * 5 + F * 36, F + 5 * F + 4, 0)
            rk, rb, _ = oracle.f3_weights("artcnn", F, kind)
            assert np.array_equal(k, rk) and np.array_equal(b, rb)
    for F in (8, 16):
        for kind, tag in enumerate(("", "-distortplus")):
            name = "fsrcnnx-f%d%s" % (F, tag)
            assert oracle.parse_model(name) == ("fsrcnnx", (F, kind))
            k, b, a = ac.model_params(name)
            assert (k.size, b.size, a.size) == (F * 25 + F * F * 9 * 4 + F * F + F * 36, F + 5 * F + 4, 5 * F)
            rk, rb, ra = oracle.f3_weights("fsrcnnx", F, kind)
            assert np.array_equal(k, rk) and np.array_equal(b, rb) and np.array_equal(a, ra)
    # "dp" is DistortPlus too, and an unknown string is ACNetLegacy GAN (Processor.cpp:186)
    assert np.array_equal(ac.model_params("FSRCNNX-dp")[0], oracle.f3_weights("fsrcnnx", 8, 1)[0])
    assert ac.model_params("no-such-model")[0].size == 4712


def test_acnet8_parameters_match_the_reference_blob(lib):
    """Every ACNet<8> variant (B4/8/18 x normal/HDN/Box/Box-HDN) resolves as the
    reference's model strings do and carries the reference's trained
    parameters, in the NHWC sizes of ACNet.hpp:79-84."""
    for blocks in (4, 8, 18):
        for kind, tag in enumerate(("", "-hdn", "-box", "-box-hdn")):
            name = "acnet-f8b%d%s" % (blocks, tag)
            assert oracle.parse_model(name) == ("acnet8", (blocks, kind))
            k, b, a = ac.model_params(name)
            assert (k.size, b.size, a.size) == (72 + 576 * blocks + 288, 8 + 8 * blocks + 4, 8 * (blocks + 1))
            rk, rb, ra = oracle.acnet8_weights(blocks, kind)
            assert np.array_equal(k, rk) and np.array_equal(b, rb) and np.array_equal(a, ra)
    # defaults: B8, and "acnet" alone is ACNet<8> B8 normal (Processor.cpp:175-184)
    assert np.array_equal(ac.model_params("acnet-hdn")[0], oracle.acnet8_weights(8, 1)[0])
    assert np.array_equal(ac.model_params("ACNet")[0], oracle.acnet8_weights(8, 0)[0])


def test_output_shape_matches_oracle_pipeline(lib):
    for (h, w, c, f) in [(17, 23, 1, 2.0), (17, 23, 3, 4.0), (10, 13, 3, 3.0), (9, 7, 1, 1.5), (5, 6, 4, 8.0)]:
        x = np.zeros((h, w, c) if c > 1 else (h, w), np.uint8)
        want = oracle.process(x, f, "acnet-legacy-hdn0", threads=1).shape
        ow, oh = ac.output_shape(w, h, c, f)
        assert (oh, ow) == tuple(want[:2])


def test_image_handles_roundtrip(lib):
    L = lib
    img = ac.ACImage()
    img.width, img.height, img.channels, img.element_type = 5, 3, 3, ac.UINT8
    assert L.ac_image_create(ctypes.byref(img)) == 0
    assert img.stride == 16 and img.ptr  # line 15 bytes aligned to 4
    data = np.arange(45, dtype=np.uint8).reshape(3, 15)
    src = ac.ACImage()
    src.width, src.height, src.channels, src.element_type = 5, 3, 3, ac.UINT8
    assert L.ac_image_from(ctypes.byref(src), data.ctypes.data) == 0
    out = np.zeros((3, 15), np.uint8)
    assert L.ac_image_to(ctypes.byref(src), out.ctypes.data, 15) == 0
    assert np.array_equal(out, data)
    view = ac.ACImage()
    assert L.ac_image_view(ctypes.byref(src), ctypes.byref(view), 1, 1, 10, 10) == 0
    assert (view.width, view.height) == (4, 2)
    assert view.ptr == src.ptr + src.stride + 3
    clone = ac.ACImage()
    assert L.ac_image_clone(ctypes.byref(src), ctypes.byref(clone)) == 0
    assert clone.ptr != src.ptr
    for i in (img, src, view, clone):
        L.ac_image_unref(ctypes.byref(i))
        assert i.ptr is None and i.hptr is None
    assert L.ac_image_ref(None, None) == -ac.AC_EINVAL
    assert L.ac_processor_ok(None) == -ac.AC_EINVAL
