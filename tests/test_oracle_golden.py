"""The CPU oracle (C restatement) against golden vectors made by the
reference's own CPU processor (tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "golden.npz"))
META = json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]


@pytest.mark.parametrize("case", META, ids=[c["name"] for c in META])
def test_oracle_bit_exact_vs_reference_generic(case):
    x = GOLD[case["name"] + "/in"]
    want = GOLD[case["name"] + "/generic"]
    got = oracle.process(x, case["factor"], case["model"], threads=2)
    assert got.shape == want.shape and got.dtype == want.dtype
    assert np.array_equal(got, want)


@pytest.mark.parametrize("case", META, ids=[c["name"] for c in META])
def test_reference_isa_spread_within_one_lsb(case):
    """The reference's SIMD backend and its Generic backend differ by at most
    1 LSB; that spread is the tolerance the CUDA path is held to."""
    g = GOLD[case["name"] + "/generic"].astype(np.float64)
    a = GOLD[case["name"] + "/auto"].astype(np.float64)
    if case["dtype"] == "float32":
        assert np.abs(g - a).max() <= 1e-4
    else:
        assert np.abs(g - a).max() <= 1


def test_point_resize_known_answer():
    """tests/core/src/ImageResizeTest.cpp:43-72 (RESIZE_POINT 2x2 -> 4x4)."""
    src = np.array([[10, 20], [30, 40]], np.uint8)
    out = oracle.resize(src, 4, 4, oracle.RESIZE_POINT)
    want = np.array([[10, 10, 20, 20], [10, 10, 20, 20], [30, 30, 40, 40], [30, 30, 40, 40]], np.uint8)
    assert np.array_equal(out, want)


def test_gray_roundtrip_within_one():
    """tests/core/src/ImageProcessTest.cpp:52-137: gray RGB -> YUV -> RGB within +-1."""
    rgb = np.full((4, 4, 3), 100, np.uint8)
    y, uv = oracle.rgb2yuv(rgb)
    back = oracle.yuv2rgb(y, uv)
    assert np.abs(back.astype(int) - 100).max() <= 1


def test_catmull_rom_x2_weights_are_exact():
    first, w = oracle.resize_coeffs(8, 16, oracle.RESIZE_CATMULL_ROM, maxtaps=5)
    even = w[4][w[4] != 0]
    odd = w[5][w[5] != 0]
    assert np.allclose(even, [-0.0234375, 0.2265625, 0.8671875, -0.0703125], atol=0)
    assert np.allclose(odd, [-0.0703125, 0.8671875, 0.2265625, -0.0234375], atol=0)
    assert first[4] == 0 and first[5] == 1


X2_CASES = [c for c in META if c["factor"] == 2.0]


@pytest.mark.parametrize("case", X2_CASES, ids=[c["name"] for c in X2_CASES])
def test_fp64_oracle_agrees_with_reference(case):
    """The FP64 twin of every network (oracle.pipeline_f64, the error
    statistics' reference) quantised at the reference's rounding points is
    within the reference's own ISA spread of the reference's output: 1 LSB
    on integer outputs, 1e-4 on f32."""
    x = GOLD[case["name"] + "/in"]
    want = GOLD[case["name"] + "/generic"]
    exact, quant = oracle.pipeline_f64(x, case["model"], threads=2)
    assert quant.shape == want.shape
    d = np.abs(quant.astype(np.float64) - want.astype(np.float64))
    if case["dtype"] == "float32":
        assert d.max() <= 1e-4
    else:
        assert d.max() <= 1
    st = oracle.error_stats(want, exact, quant)
    assert st["frac_within_1lsb"] == 1.0


LEGACY_CASES = [c for c in META if "legacy" in c["model"]]


@pytest.mark.parametrize("case", LEGACY_CASES, ids=[c["name"] for c in LEGACY_CASES])
def test_neon_order_port_within_reference_isa_spread(case):
    """The 4-lane restatement of the reference's NEON backend (the timed CPU
    baseline on the aarch64 GPU host) differs from the reference's Generic
    output by at most what the reference's own SIMD backend does."""
    x = GOLD[case["name"] + "/in"]
    want = GOLD[case["name"] + "/generic"].astype(np.float64)
    got = oracle.process(x, case["factor"], case["model"], threads=2, order="neon").astype(np.float64)
    if case["dtype"] == "float32":
        assert np.abs(got - want).max() <= 1e-4
    else:
        assert np.abs(got - want).max() <= 1
