"""ACNet<8> (the reference CLI's default family, acnet-f8b{4,8,18}[-hdn][-box])
on the GPU against the oracle (GPU required).

Tolerances: the plain FP32 form holds the ACNetLegacy gate (integer outputs
never more than 1 LSB from the reference CPU processor; f32 within 1e-4).
The tensor-core forms (B4 / B8: every layer in the persistent quad kernel,
layer 0 and the tail with split 16-bit weights, activations in 16 bits inside
the tile; B18: two layers per launch, FP32 head and upscale, 16-bit maps
between launches): FP16 PSNR >= 50 dB against the FP64 oracle and u8 within
2 LSB of the reference CPU output (>= 99 % of pixels within 1); BF16 PSNR >=
40 dB and within 8 LSB; f32 outputs within 2e-3 (FP16) / 2e-2 (BF16).  RGB(A)
through the fused colour path: the ACNetLegacy FP16 RGB gate, within 6 LSB and
>= 99 % of values within 1 (RGBA un-premultiplies by alpha, which scales a
1-LSB luma difference up where alpha is small).
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


@pytest.mark.parametrize("model", ["acnet-f8b4-hdn", "acnet-f8b8"])
@pytest.mark.parametrize("c", [3, 4])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
def test_acnet8_quad_rgb_vs_oracle(model, c, dtype):
    """B4 / B8 RGB(A) x2: split, every CNN layer, chroma resample and merge in
    the one persistent quad kernel, against the reference CPU pipeline."""
    x = synthetic.rgb_u8(53, 101, seed=21, alpha=(c == 4))
    if dtype == "uint16":
        x = (x.astype(np.uint16) * 257).astype(np.uint16)
    elif dtype == "float32":
        x = (x.astype(np.float32) / 255.0).astype(np.float32)
    got = run(model, x, 2.0, "fp16")
    want = oracle.process(x, 2.0, model)
    assert got.shape == want.shape
    if dtype == "float32":
        assert np.abs(got - want).max() <= 3e-3
        return
    lsb = 1 if dtype == "uint8" else 257
    d = np.abs(got.astype(np.int64) - want.astype(np.int64))
    assert d.max() <= 6 * lsb and (d <= lsb).mean() >= 0.99, (d.max(), (d <= lsb).mean())


@pytest.mark.parametrize("c", [3, 4])
@pytest.mark.parametrize("form", ["fp16", "bf16"])
def test_acnet8_quad_fused_colour_matches_unfused(c, form, monkeypatch):
    """The fused RGB(A) kernel equals split + quad luma kernel + merge bit for bit."""
    x = synthetic.rgb_u8(61, 83, seed=5, alpha=(c == 4))
    outs = []
    for fused in ("1", "0"):
        monkeypatch.setenv("AC_GB300_FUSED", fused)
        p = ac.Processor("cuda", 0, "acnet-f8b8-hdn", precision=form)
        outs.append(p.process(x, 2.0))
        assert p.ok(), p.error()
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("model", ["acnet-f8b4", "acnet-f8b8-box-hdn"])
@pytest.mark.parametrize("c", [1, 3])
def test_acnet8_quad_batch_equals_single(model, c):
    """One launch over a batch of uneven images gives each image the bytes of
    its own launch (direct launch, graph capture, graph replay)."""
    import torch
    sizes = [(37, 53), (64, 64), (95, 140), (1, 7), (44, 44), (47, 93)]
    imgs = [synthetic.luma(h, w, np.uint8, seed=h + w) if c == 1 else synthetic.rgb_u8(h, w, seed=h + w) for h, w in sizes]
    p = ac.Processor("cuda", 0, model, precision="fp16")
    singles = [p.process(x, 2.0) for x in imgs]
    assert p.ok(), p.error()
    srcs = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in imgs]
    dsts = [torch.empty((2 * x.shape[0], 2 * x.shape[1]) + x.shape[2:], dtype=torch.uint8, device="cuda") for x in imgs]
    for _ in range(3):
        p.process_batch_device(srcs, dsts, 2.0)
        assert p.ok(), p.error()
        for d, want in zip(dsts, singles):
            assert np.array_equal(d.cpu().numpy(), want)


def test_acnet8_quad_close_to_layer_pair_form(monkeypatch):
    """B8 through the quad kernel and through the two-layers-per-launch form
    (AC_GB300_TC_KERNEL=3 keeps ACNet<8> on the latter) agree within the
    tensor-core tolerance."""
    x = synthetic.luma(90, 160, np.uint8, seed=2)
    quad = run("acnet-f8b8-hdn", x, 2.0, "fp16")
    monkeypatch.setenv("AC_GB300_TC_KERNEL", "3")
    pair = run("acnet-f8b8-hdn", x, 2.0, "fp16")
    assert np.abs(quad.astype(int) - pair.astype(int)).max() <= 2


@pytest.mark.parametrize("form", ["fp16", "bf16"])
@pytest.mark.parametrize("c", [1, 3, 4])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
def test_acnet8_b8_split_gives_identical_bytes(form, c, dtype, monkeypatch):
    """ACNet<8> B8 split in two quad-kernel launches at layer 5 (the head
    stores block 4's activations after PReLU in a 16-bit map) against the
    whole network in one launch: the same bytes, one image and a batch of
    sizes with tiles at every edge and images smaller than a tile."""
    torch = pytest.importorskip("torch")
    sizes = [(131, 150), (1, 1), (7, 93), (54, 52), (200, 45)]
    imgs = []
    for h, w in sizes:
        x = synthetic.rgb_u8(h, w, seed=h + w, alpha=(c == 4)) if c > 1 else synthetic.luma(h, w, np.uint8, seed=h + w)
        if dtype == "uint16":
            x = (x.astype(np.uint16) * 257).astype(np.uint16)
        elif dtype == "float32":
            x = (x.astype(np.float32) / 255.0).astype(np.float32)
        imgs.append(np.ascontiguousarray(x))
    srcs = [torch.from_numpy(x).cuda() for x in imgs]
    outs = {}
    for depth in ("9", "5"):
        monkeypatch.setenv("AC_GB300_FUSION_DEPTH", depth)
        p = ac.Processor("cuda", 0, "acnet-f8b8-hdn", precision=form)
        single = torch.empty((2 * sizes[0][0], 2 * sizes[0][1]) + imgs[0].shape[2:], dtype=srcs[0].dtype, device="cuda")
        p.process_device(srcs[0], single, 2.0)
        dsts = [torch.empty((2 * s.shape[0], 2 * s.shape[1]) + tuple(s.shape[2:]), dtype=s.dtype, device="cuda") for s in srcs]
        p.process_batch_device(srcs, dsts, 2.0)
        assert p.ok(), p.error()
        outs[depth] = [single.cpu().numpy()] + [d.cpu().numpy() for d in dsts]
    for a, b in zip(outs["9"], outs["5"]):
        assert np.array_equal(a, b)
