"""ArtCNN<16/32> and FSRCNNX<8/16> (the reference's other CNN families) on the
GPU against the oracle (GPU required).

Plain FP32 form: integer outputs never more than 1 LSB from the reference CPU
processor, f32 outputs within 1e-4.  Tensor-core form (ArtCNN<16/32>,
FSRCNNX<16>: FP16/BF16 3x3 layers, the upscale with split 16-bit weights, FP32
head; FSRCNNX<8>: FP16/BF16 3x3 layers two per launch, FP32 head and upscale;
16-bit maps between launches): FP16
u8 outputs within 2 LSB on >= 99 % of pixels and never more than 6 LSB off,
f32 within 5e-3; BF16 within 16 LSB, f32 within 3e-2; u16 the u8 gates in
units of 257 (1/255 of the range).
"""
import numpy as np
import pytest

import anime4kcpp_gb300 as ac
import oracle
from anime4kcpp_gb300 import synthetic

pytestmark = pytest.mark.gpu

VARIANTS = ["artcnn-c4f16", "artcnn-c4f16-dn", "artcnn-c4f16-ds", "artcnn-c4f32", "artcnn-c4f32-dn", "artcnn-c4f32-ds",
            "fsrcnnx-f8", "fsrcnnx-f8-dp", "fsrcnnx-f16", "fsrcnnx-f16-dp"]


@pytest.fixture(scope="module", autouse=True)
def built():
    from anime4kcpp_gb300 import build
    build.build()
    oracle.build()


def run(model, x, factor, form="fp32"):
    p = ac.Processor("cuda", 0, model, precision=form)
    assert p.ok(), p.error()
    out = p.process(x, factor)
    assert p.ok(), p.error()
    return out


@pytest.mark.parametrize("model", VARIANTS)
def test_f3_every_variant_u8(model):
    x = synthetic.luma(45, 77, np.uint8, seed=4)
    d = np.abs(run(model, x, 2.0).astype(int) - oracle.process(x, 2.0, model).astype(int))
    assert d.max() <= 1 and (d > 0).mean() <= 1e-3


@pytest.mark.parametrize("model", ["artcnn-c4f32-ds", "fsrcnnx-f16"])
@pytest.mark.parametrize("dtype", ["uint16", "float32"])
@pytest.mark.parametrize("shape", [(37, 70), (1, 33), (29, 1), (2, 3)])
def test_f3_types_and_sizes(model, dtype, shape):
    h, w = shape
    x = synthetic.f32_luma_uniform(h, w, seed=h + w) if dtype == "float32" else synthetic.luma(h, w, np.uint16, seed=h + w)
    got = run(model, x, 2.0)
    want = oracle.process(x, 2.0, model)
    if dtype == "float32":
        assert np.abs(got - want).max() <= 1e-4
    else:
        assert np.abs(got.astype(int) - want.astype(int)).max() <= 1


@pytest.mark.parametrize("model,factor,c", [("artcnn-c4f16", 2.0, 3), ("fsrcnnx-f8", 4.0, 3), ("artcnn-c4f32-dn", 2.0, 4)])
def test_f3_rgb_pipeline(model, factor, c):
    x = synthetic.rgb_u8(31, 45, seed=6, alpha=(c == 4))
    got = run(model, x, factor)
    want = oracle.process(x, factor, model)
    assert got.shape == want.shape
    assert np.abs(got.astype(int) - want.astype(int)).max() <= 1


def test_fsrcnnx_f8_tensor_core_form_close_to_fp32_form(monkeypatch):
    """FSRCNNX<8>'s tensor-core form against its plain FP32 form (FP16 requested
    with the tensor-core form switched off runs the FP32 pipeline)."""
    x = synthetic.luma(90, 160, np.uint8, seed=8)
    tc = run("fsrcnnx-f8", x, 2.0, "fp16")
    monkeypatch.setenv("AC_GB300_ARNET_TC", "0")
    fp32 = run("fsrcnnx-f8", x, 2.0, "fp16")
    assert np.array_equal(fp32, run("fsrcnnx-f8", x, 2.0, "fp32"))
    assert np.abs(tc.astype(int) - fp32.astype(int)).max() <= 6


@pytest.mark.parametrize("form", ["fp16", "bf16"])
@pytest.mark.parametrize("model", ["artcnn-c4f16", "artcnn-c4f16-dn", "artcnn-c4f32", "artcnn-c4f32-ds", "fsrcnnx-f16",
                                   "fsrcnnx-f16-dp", "fsrcnnx-f8", "fsrcnnx-f8-dp"])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
def test_f3_tc_vs_oracle(model, form, dtype):
    h, w = 67, 95  # several 30x30 tiles with ragged edges
    x = synthetic.f32_luma_uniform(h, w, seed=5) if dtype == "float32" else synthetic.luma(h, w, np.dtype(dtype), seed=5)
    got = run(model, x, 2.0, form)
    want = oracle.process(x, 2.0, model)
    if dtype == "float32":
        assert np.abs(got - want).max() <= (5e-3 if form == "fp16" else 3e-2)
        return
    lsb = 1 if dtype == "uint8" else 257  # u16: the u8 gates in units of 1/255
    d = np.abs(got.astype(np.int64) - want.astype(np.int64))
    if form == "fp16":
        assert (d <= 2 * lsb).mean() >= 0.99 and d.max() <= 6 * lsb, (d.max(), (d <= 2 * lsb).mean())
    else:
        assert d.max() <= 16 * lsb, d.max()


@pytest.mark.parametrize("shape", [(1, 40), (45, 1), (30, 30), (31, 31), (2, 3)])
def test_f3_tc_odd_sizes(shape):
    h, w = shape
    x = synthetic.luma(h, w, np.uint8, seed=h * 100 + w)
    for model in ("artcnn-c4f32", "fsrcnnx-f16", "fsrcnnx-f8"):
        d = np.abs(run(model, x, 2.0, "fp16").astype(int) - oracle.process(x, 2.0, model).astype(int))
        assert d.max() <= 6


def test_f3_tc_rgb_x4():
    x = synthetic.rgb_u8(40, 56, seed=12)
    got = run("artcnn-c4f16", x, 4.0, "fp16")
    want = oracle.process(x, 4.0, "artcnn-c4f16")
    d = np.abs(got.astype(int) - want.astype(int))
    assert got.shape == want.shape and d.max() <= 8 and (d <= 2).mean() >= 0.99
