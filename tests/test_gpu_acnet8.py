"""ACNet<8> (the reference CLI's default family, acnet-f8b{4,8,18}[-hdn][-box])
on the GPU against the oracle (GPU required).

Tolerances: the plain FP32 form holds the ACNetLegacy gate (integer outputs
never more than 1 LSB from the reference CPU processor; f32 within 1e-4).
The tensor-core forms (FP16 / BF16 8->8 layers, FP32 head and upscale, 16-bit
maps between layers): FP16 PSNR >= 50 dB against the FP64 oracle and u8 within
2 LSB of the reference CPU output (>= 99 % of pixels within 1); BF16 PSNR >=
40 dB and within 8 LSB; f32 outputs within 2e-3 (FP16) / 2e-2 (BF16).
"""
import numpy as np
import pytest

import anime4kcpp_gb300 as ac
import oracle
from anime4kcpp_gb300 import synthetic

pytestmark = pytest.mark.gpu

VARIANTS = ["acnet-f8b%d%s" % (b, t) for b in (4, 8, 18) for t in ("", "-hdn", "-box", "-box-hdn")]


@pytest.fixture(scope="module", autouse=True)
def built():
    from anime4kcpp_gb300 import build
    build.build()
    oracle.build()


def psnr(got, ref64, scale):
    err = got.astype(np.float64) / scale - np.clip(ref64, 0.0, 1.0)
    mse = np.mean(err * err)
    return 99.0 if mse == 0 else 10 * np.log10(1.0 / mse)


def run(model, x, factor, form):
    p = ac.Processor("cuda", 0, model, precision=form)
    assert p.ok(), p.error()
    out = p.process(x, factor)
    assert p.ok(), p.error()
    return out


@pytest.mark.parametrize("model", VARIANTS)
def test_acnet8_fp32_every_variant(model):
    x = synthetic.luma(45, 77, np.uint8, seed=3)
    d = np.abs(run(model, x, 2.0, "fp32").astype(int) - oracle.process(x, 2.0, model).astype(int))
    assert d.max() <= 1 and (d > 0).mean() <= 1e-3


@pytest.mark.parametrize("dtype", ["uint16", "float32"])
@pytest.mark.parametrize("shape", [(40, 70), (1, 33), (29, 1)])
def test_acnet8_fp32_types_and_sizes(dtype, shape):
    h, w = shape
    x = synthetic.f32_luma_uniform(h, w, seed=h + w) if dtype == "float32" else synthetic.luma(h, w, np.uint16, seed=h + w)
    got = run("acnet-f8b8-hdn", x, 2.0, "fp32")
    want = oracle.process(x, 2.0, "acnet-f8b8-hdn")
    if dtype == "float32":
        assert np.abs(got - want).max() <= 1e-4
    else:
        assert np.abs(got.astype(int) - want.astype(int)).max() <= 1


@pytest.mark.parametrize("c,factor", [(3, 2.0), (4, 2.0), (3, 4.0), (3, 3.0)])
def test_acnet8_fp32_rgb_pipeline(c, factor):
    x = synthetic.rgb_u8(37, 53, seed=9, alpha=(c == 4))
    got = run("acnet-f8b4-hdn", x, factor, "fp32")
    want = oracle.process(x, factor, "acnet-f8b4-hdn")
    assert got.shape == want.shape
    assert np.abs(got.astype(int) - want.astype(int)).max() <= 1


@pytest.mark.parametrize("form", ["fp16", "bf16"])
@pytest.mark.parametrize("model", ["acnet-f8b4", "acnet-f8b8-hdn", "acnet-f8b18-box", "acnet-f8b18-box-hdn"])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
def test_acnet8_tc_vs_oracle(model, form, dtype):
    h, w = 67, 131  # several 62x30 tiles with ragged edges
    x = synthetic.f32_luma_uniform(h, w, seed=5) if dtype == "float32" else synthetic.luma(h, w, np.dtype(dtype), seed=5)
    got = run(model, x, 2.0, form)
    ref32 = oracle.process(x, 2.0, model)
    if dtype == "float32":
        assert np.abs(got - ref32).max() <= (2e-3 if form == "fp16" else 2e-2)
        return
    ref64 = oracle.process_f64(x, model)
    scale = 255.0 if dtype == "uint8" else 65535.0
    p = psnr(got, ref64, scale)
    assert p >= (50.0 if form == "fp16" else 40.0), p
    if dtype == "uint8":
        d = np.abs(got.astype(int) - ref32.astype(int))
        assert d.max() <= (2 if form == "fp16" else 8), d.max()
        if form == "fp16":
            assert (d <= 1).mean() >= 0.99


@pytest.mark.parametrize("shape", [(1, 40), (45, 1), (30, 62), (31, 63), (2, 2), (1, 1)])
def test_acnet8_tc_odd_sizes(shape):
    h, w = shape
    x = synthetic.luma(h, w, np.uint8, seed=h * 100 + w)
    d = np.abs(run("acnet-f8b8", x, 2.0, "fp16").astype(int) - oracle.process(x, 2.0, "acnet-f8b8").astype(int))
    assert d.max() <= 2


def test_acnet8_tc_rgb_x4():
    x = synthetic.rgb_u8(40, 56, seed=12)
    got = run("acnet-f8b8-hdn", x, 4.0, "fp16")
    want = oracle.process(x, 4.0, "acnet-f8b8-hdn")
    d = np.abs(got.astype(int) - want.astype(int))
    assert got.shape == want.shape and d.max() <= 3 and (d <= 1).mean() >= 0.99


def test_acnet8_tc_and_fp32_forms_close(monkeypatch):
    x = synthetic.luma(90, 160, np.uint8, seed=2)
    tc = run("acnet-f8b18", x, 2.0, "fp16")
    monkeypatch.setenv("AC_GB300_ARNET_TC", "0")
    fp32 = run("acnet-f8b18", x, 2.0, "fp16")  # FP16 requested, tensor-core form disabled: the FP32 pipeline
    assert np.abs(tc.astype(int) - fp32.astype(int)).max() <= 2
