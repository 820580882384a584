"""ArtCNN<16/32> and FSRCNNX<8/16> (the reference's other CNN families) on the
GPU against the oracle (GPU required).

These families run a plain FP32 layer pipeline in every precision form; the
tolerance is the plain form's: integer outputs never more than 1 LSB from the
reference CPU processor, f32 outputs within 1e-4.
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


def test_f3_every_form_runs_the_fp32_pipeline():
    x = synthetic.luma(40, 52, np.uint8, seed=8)
    outs = [run("artcnn-c4f16", x, 2.0, form) for form in ("fp32", "fp16", "bf16")]
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
