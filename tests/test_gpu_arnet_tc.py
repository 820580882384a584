"""ARNet<8> tensor-core form (FP16/BF16 8->8 layers on tcgen05, two per launch,
FP32 head and upscale, 16-bit maps between launches) against the oracle (GPU
required).

Tolerances: u8 outputs within 1 LSB of the reference CPU processor and PSNR
>= 50 dB against the FP64 oracle; u16 outputs PSNR >= 80 dB (FP16) / 60 dB
(BF16) against the FP64 oracle; f32 outputs within 2e-3 (FP16) / 2e-2 (BF16).
"""
import numpy as np
import pytest

import anime4kcpp_gb300 as ac
import oracle
from anime4kcpp_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from anime4kcpp_gb300 import build
    build.build()
    oracle.build()


def psnr(got, ref64, scale):
    err = got.astype(np.float64) / scale - np.clip(ref64, 0.0, 1.0)
    mse = np.mean(err * err)
    return 99.0 if mse == 0 else 10 * np.log10(1.0 / mse)


@pytest.mark.parametrize("form", ["fp16", "bf16"])
@pytest.mark.parametrize("model", ["arnet-b8", "arnet-hdn-b16", "arnet-box-b32", "arnet-box-hdn-b64"])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
def test_arnet_tc_vs_oracle(model, form, dtype):
    h, w = 67, 131  # several 62x30 tiles with ragged edges
    if dtype == "float32":
        x = synthetic.f32_luma_uniform(h, w, seed=5)
    else:
        x = synthetic.luma(h, w, np.dtype(dtype), seed=5)
    p = ac.Processor("cuda", 0, model, precision=form)
    got = p.process(x, 2.0)
    assert p.ok(), p.error()
    ref32 = oracle.process(x, 2.0, model)
    if dtype == "float32":
        assert np.abs(got - ref32).max() <= (2e-3 if form == "fp16" else 2e-2)
        return
    ref64 = oracle.process_f64(x, model)
    scale = 255.0 if dtype == "uint8" else 65535.0
    if dtype == "uint8":
        assert np.abs(got.astype(int) - ref32.astype(int)).max() <= 1
        assert psnr(got, ref64, scale) >= 50.0
    else:
        assert psnr(got, ref64, scale) >= (80.0 if form == "fp16" else 60.0)


@pytest.mark.parametrize("shape", [(1, 40), (45, 1), (30, 62), (31, 63), (2, 2)])
def test_arnet_tc_odd_sizes(shape):
    h, w = shape
    x = synthetic.luma(h, w, np.uint8, seed=h * 100 + w)
    p = ac.Processor("cuda", 0, "arnet-b8", precision="fp16")
    got = p.process(x, 2.0)
    assert p.ok(), p.error()
    assert np.abs(got.astype(int) - oracle.process(x, 2.0, "arnet-b8").astype(int)).max() <= 1


def test_arnet_tc_x4_video_recipe():
    """10-bit luma shifted by 6, x4 as two chained x2 passes, FP16 form."""
    y10 = synthetic.luma(68, 120, np.uint16, seed=11, noise=4.0, bits=10)
    x = (y10 << 6).astype(np.uint16)
    p = ac.Processor("cuda", 0, "arnet-b8", precision="fp16")
    got = p.process(x, 4.0)
    assert p.ok(), p.error()
    want = oracle.process(x, 4.0, "arnet-b8")
    d = np.abs((got >> 6).astype(int) - (want >> 6).astype(int))
    assert d.max() <= 1 and (d == 0).mean() >= 0.98  # within 1 LSB of the 10-bit value


def test_arnet_tc_matches_fp32_pipeline_closely(monkeypatch):
    x = synthetic.rgb_u8(90, 160, seed=2)
    p = ac.Processor("cuda", 0, "arnet-b8", precision="fp16")
    tc = p.process(x, 2.0)
    monkeypatch.setenv("AC_GB300_ARNET_TC", "0")
    q = ac.Processor("cuda", 0, "arnet-b8", precision="fp16")
    fp32 = q.process(x, 2.0)
    assert np.abs(tc.astype(int) - fp32.astype(int)).max() <= 2


@pytest.mark.parametrize("factor", [2.0, 4.0])
@pytest.mark.parametrize("model", ["arnet-b8", "acnet-f8b18-hdn", "acnet-f8b8-hdn", "artcnn-c4f16", "artcnn-c4f32-ds",
                                   "fsrcnnx-f16", "fsrcnnx-f8-dp"])
def test_layered_tc_batch_equals_single(model, factor):
    """Tensor-core forms over a batch of uneven single-channel images: ARNet,
    ACNet<8> B18, ArtCNN and FSRCNNX run every layer (or layer pair) as one
    launch over all images, ACNet<8> B8 the whole pass as the split network's
    two quad-kernel launches (B4: one); each image gets the bytes of its own
    per-image run (x4: two chained batched x2 passes)."""
    import torch
    sizes = [(67, 131), (30, 62), (1, 40), (45, 1), (90, 33)]
    imgs = [synthetic.luma(h, w, np.uint16, seed=h * 7 + w, noise=4.0, bits=10) << 6 for h, w in sizes]
    imgs = [x.astype(np.uint16) for x in imgs]
    p = ac.Processor("cuda", 0, model, precision="fp16")
    singles = [p.process(x, factor) for x in imgs]
    assert p.ok(), p.error()
    f = int(factor)
    srcs = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in imgs]
    dsts = [torch.empty((f * x.shape[0], f * x.shape[1]), dtype=torch.uint16, device="cuda") for x in imgs]
    l0 = ac.launch_count()
    p.process_batch_device(srcs, dsts, factor)
    assert p.ok(), p.error()
    launches = ac.launch_count() - l0
    # head, the layers (two per launch for the 8-channel families, one for ArtCNN / FSRCNNX<16>), upscale;
    # or the quad kernel's launches (ACNet<8> B8: the split network's head and tail)
    layers = {"arnet-b8": 8 + 2, "acnet-f8b18-hdn": 9 + 2, "acnet-f8b8-hdn": 2, "artcnn-c4f16": 5 + 2,
              "artcnn-c4f32-ds": 5 + 2, "fsrcnnx-f16": 4 + 2, "fsrcnnx-f8-dp": 2 + 2}[model]
    assert launches == layers * (2 if factor == 4.0 else 1)
    for d, want in zip(dsts, singles):
        assert np.array_equal(d.cpu().numpy(), want)
