"""The ``pyac``-shaped module (binding/python/src/Binding.cpp:15-190): its
layout, defaults and lists on the CPU; on the GPU, that its default processor
is the library's ``acnet-f8b8-hdn`` path and that it raises like the
reference on a bad call."""
import json
import os

import numpy as np
import pytest

import anime4kcpp_gb300 as ac
import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def pyac():
    from anime4kcpp_gb300 import build
    build.build()
    from anime4kcpp_gb300 import pyac
    return pyac


def test_core_layout(pyac):
    core = pyac.core
    for name in ("Processor", "resize", "ResizeModes"):
        assert hasattr(core, name)
    # Binding.cpp:78-96: seventeen modes, exported onto core
    names = [m.name for m in core.ResizeModes]
    assert names[0] == "RESIZE_POINT" and names[-1] == "RESIZE_BILINEAR" and len(names) == 17
    for m in core.ResizeModes:
        assert getattr(core, m.name) is m and int(m) == getattr(ac, m.name)
    assert (core.Processor.CPU, core.Processor.OpenCL, core.Processor.CUDA) == (0, 1, 2)
    # def_property_readonly_static: readable on the class itself
    info = core.Processor.InfoList
    assert isinstance(info, tuple) and all(isinstance(s, str) for s in info)


def test_model_list_matches_the_reference_listing(pyac):
    ref = json.load(open(os.path.join(HERE, "golden", "model_list.json")))
    ours = pyac.specs.ModelList
    assert [m["name"] for m in ours] == [m["name"] for m in ref]
    assert [m["parameter_count"] for m in ours] == [m["parameter_count"] for m in ref]
    # third-party models carry their version, author and homepage
    for key in ("version", "author", "homepage"):
        assert [m[key] for m in ours] == [m[key] for m in ref], key
    for m in ours:
        assert set(m) == {"name", "description", "parameter_count", "version", "author", "homepage"}
        assert m["description"]


def test_model_list_names_select_their_own_networks(pyac):
    """Every listed string parses to the family its name says
    (Processor.cpp:26-187), not to the fallback default."""
    for m in pyac.specs.ModelList:
        family, _ = oracle.parse_model(m["name"])
        head = m["name"].split("-")[0]
        expect = {"acnet": "acnet_legacy" if "legacy" in m["name"] else "acnet8",
                  "arnet": "arnet", "artcnn": "artcnn", "fsrcnnx": "fsrcnnx"}[head]
        assert family == expect, m["name"]


def test_processor_list(pyac):
    assert [p["name"] for p in pyac.specs.ProcessorList] == ["cuda"]


def test_default_processor_without_a_gpu_fails_loudly(pyac):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = pyac.core.Processor()
    assert not p.ok() and p.error()
    with pytest.raises(RuntimeError):
        p(np.zeros((4, 4), np.uint8))


@pytest.mark.gpu
def test_default_processor_is_acnet8_b8_hdn(pyac):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (61, 83, 3), dtype=np.uint8)
    p = pyac.core.Processor()
    assert p.ok(), p.error()
    assert str(p) == p.name() and str(p)  # the device's name, as Processor::name
    out = p(img)
    ref = ac.Processor("cuda", 0, "acnet-f8b8-hdn")(img, 2.0)
    assert out.shape == (122, 166, 3) and np.array_equal(out, ref)
    # positional arguments as the reference takes them
    q = pyac.core.Processor("cuda", 0, "acnet-legacy-hdn0")
    assert np.array_equal(q.process(img, 2.0), ac.Processor("cuda", 0, "acnet-legacy-hdn0").process(img, 2.0))


@pytest.mark.gpu
def test_resize_signature(pyac):
    rng = np.random.default_rng(6)
    img = rng.integers(0, 256, (40, 50, 3), dtype=np.uint8)
    a = pyac.core.resize(img, (100, 80))
    b = pyac.core.resize(img, None, 2.0, 2.0, pyac.core.RESIZE_BILINEAR)
    assert a.shape == b.shape == (80, 100, 3) and np.array_equal(a, b)
    c = pyac.core.resize(img, None, 0.5, 0.5, pyac.core.ResizeModes.RESIZE_CATMULL_ROM)
    assert np.array_equal(c, ac.resize(img, None, 0.5, 0.5, ac.RESIZE_CATMULL_ROM))
